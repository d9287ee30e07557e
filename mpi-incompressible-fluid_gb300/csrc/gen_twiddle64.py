"""Writes twiddle64.cuh: cos and sin of 2*pi*k/64 (k = 0..63) as correctly
rounded double literals, for the compile-time twiddles of the in-register DFTs.

    python gen_twiddle64.py > twiddle64.cuh
"""
from mpmath import cos, mp, pi, sin

mp.dps = 50


def lit(v):
    f = float(v)
    return "0.0" if abs(f) < 1e-30 else repr(f)


print("// cos and sin of 2*pi*k/64, k = 0..63, correctly rounded to double; generated by")
print("// gen_twiddle64.py. The in-register DFTs index them with compile-time k.")
print("#pragma once")
print("namespace mifgpu {")
print("__device__ constexpr double kCos64[64] = {" + ", ".join(lit(cos(2 * pi * k / 64)) for k in range(64)) + "};")
print("__device__ constexpr double kSin64[64] = {" + ", ".join(lit(sin(2 * pi * k / 64)) for k in range(64)) + "};")
print("}  // namespace mifgpu")
