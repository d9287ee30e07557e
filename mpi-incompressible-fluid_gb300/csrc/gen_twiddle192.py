"""Writes twiddle192.cuh: cos and sin of 2*pi*k/192 (k = 0..191) as correctly
rounded double literals, for the compile-time twiddles of the in-register DFTs.
192 = 3 * 64 holds the roots of unity of every transform length the register
path builds from radix-2 steps on a radix-2 or radix-3 base (2..64, 3..192).

    python gen_twiddle192.py > twiddle192.cuh
"""
from mpmath import cos, mp, pi, sin

mp.dps = 50


def lit(v):
    f = float(v)
    return "0.0" if abs(f) < 1e-30 else repr(f)


print("// cos and sin of 2*pi*k/192, k = 0..191, correctly rounded to double; generated by")
print("// gen_twiddle192.py. The in-register DFTs index them with compile-time k.")
print("#pragma once")
print("namespace mifgpu {")
print("__device__ constexpr double kCos192[192] = {" + ", ".join(lit(cos(2 * pi * k / 192)) for k in range(192)) + "};")
print("__device__ constexpr double kSin192[192] = {" + ", ".join(lit(sin(2 * pi * k / 192)) for k in range(192)) + "};")
print("}  // namespace mifgpu")
