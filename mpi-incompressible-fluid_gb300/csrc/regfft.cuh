// Register-resident line transforms for FFT lengths 64..1024 that are powers
// of two, and 384 and 768 (3 x 2^k).
//
// A complex FFT of length L = N1 * N2 is done in two register passes with one
// shared-memory transpose between them (Cooley-Tukey, "four step"): N2
// threads own one line pair; thread t first transforms the N1 elements
// x[n1*N2 + t] in registers, multiplies by W_L^(t k1), writes them transposed,
// then transforms N1/N2 columns of length N2 and holds X[k1 + N1*k2]. The
// in-register DFTs are recursive radix-2 down to a 2- or 3-point base with
// compile-time twiddles, so no index arithmetic or twiddle loads remain
// inside them.
//
// The DCT-I / R2HC / HC2R pre- and post-processing of the shared-memory
// engine (poisson_impl.cuh) is folded into the first pass's reads and the
// final store, and the z sweep's eigenvalue product into the second FFT's
// reads. Rows hold only the line's n points; the even extension of DCT-I is
// read by reflection.
#pragma once

#include "common.cuh"
#include "fft.cuh"
#include "twiddle192.cuh"

namespace mifgpu {

// o * exp(SIGN * 2 pi i k / N) with k a compile-time constant after unrolling.
template <typename T2, int N, int SIGN>
__device__ __forceinline__ T2 rot(T2 o, int k) {
  using T = decltype(o.x);
  if (k == 0) return o;
  if (4 * k == N) {  // i * SIGN
    T2 r;
    r.x = T(-SIGN) * o.y;
    r.y = T(SIGN) * o.x;
    return r;
  }
  static_assert(192 % N == 0, "root of unity in the 192-entry table");
  const T c = T(kCos192[k * (192 / N)]);
  const T s = T(SIGN) * T(kSin192[k * (192 / N)]);
  T2 r;
  r.x = o.x * c - o.y * s;
  r.y = o.x * s + o.y * c;
  return r;
}

// In-place DFT of N register values (natural order in and out), exponent sign SIGN.
template <typename T2, int N, int SIGN>
struct RegDft {
  __device__ __forceinline__ static void run(T2 *x) {
    T2 e[N / 2], o[N / 2];
#pragma unroll
    for (int k = 0; k < N / 2; ++k) {
      e[k] = x[2 * k];
      o[k] = x[2 * k + 1];
    }
    RegDft<T2, N / 2, SIGN>::run(e);
    RegDft<T2, N / 2, SIGN>::run(o);
#pragma unroll
    for (int k = 0; k < N / 2; ++k) {
      const T2 t = rot<T2, N, SIGN>(o[k], k);
      x[k] = cadd(e[k], t);
      x[k + N / 2] = csub(e[k], t);
    }
  }
};
// 3-point base: X_k = x0 + x1 w^k + x2 w^(2k), w = exp(SIGN 2 pi i / 3).
template <typename T2, int SIGN>
struct RegDft<T2, 3, SIGN> {
  __device__ __forceinline__ static void run(T2 *x) {
    using T = decltype(x[0].x);
    const T c = T(-0.5), s = T(SIGN) * T(kSin192[64]);  // cos, sin of 2 pi / 3
    const T2 a = x[0], b = x[1], d = x[2];
    const T sx = b.x + d.x, sy = b.y + d.y, dx = b.x - d.x, dy = b.y - d.y;
    const T mx = a.x + c * sx, my = a.y + c * sy;
    x[0].x = a.x + sx;
    x[0].y = a.y + sy;
    x[1].x = mx - s * dy;
    x[1].y = my + s * dx;
    x[2].x = mx + s * dy;
    x[2].y = my - s * dx;
  }
};
template <typename T2, int SIGN>
struct RegDft<T2, 2, SIGN> {
  __device__ __forceinline__ static void run(T2 *x) {
    const T2 t = x[1];
    x[1] = csub(x[0], t);
    x[0] = cadd(x[0], t);
  }
};

// Row stride (complex elements) for a pair: the N1 x (N2+1) padded transpose
// plus two, so consecutive rows fall in different banks and every row starts
// 16-byte aligned (16-byte stores of two complex values).
template <int N1, int N2>
struct RegShape {
  static constexpr int L = N1 * N2;
  static constexpr int ROW = N1 * (N2 + 1) + 2;
};

}  // namespace mifgpu
