// Shared-memory complex FFT engine for batches of lines (sm_103a).
//
// A CTA holds P independent complex sequences of length L in shared memory,
// one row of LS = L + 1 elements each (the extra element staggers rows across
// banks). The transform is a mixed-radix Stockham sweep: every stage reads
// the R inputs of each butterfly into registers, synchronises, and writes the
// R outputs in auto-sorted order, so one buffer suffices and the result ends
// in natural order. Radices 2, 3, 4, 5, 7, 8, 11, 13 have register
// butterflies; a length with any other prime factor is done as one direct DFT.
//
// Twiddles come from a per-length table tw[e] = exp(-2 pi i e / L) computed on
// the host in long double; the inverse direction conjugates them.
#pragma once

#include "common.cuh"

namespace mifgpu {

template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename T2>
__device__ __forceinline__ T2 cadd(T2 a, T2 b) {
  T2 r;
  r.x = a.x + b.x;
  r.y = a.y + b.y;
  return r;
}
template <typename T2>
__device__ __forceinline__ T2 csub(T2 a, T2 b) {
  T2 r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}
// FP32 complex add and subtract as one packed FP32x2 instruction each (each
// lane rounds as the scalar operation would: a - b is fma(b, -1, a), one
// rounding of the exact difference).
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// a * (i * sign)
template <typename T2>
__device__ __forceinline__ T2 cmul_isign(T2 a, int sign) {
  T2 r;
  if (sign < 0) {
    r.x = a.y;
    r.y = -a.x;
  } else {
    r.x = -a.y;
    r.y = a.x;
  }
  return r;
}
template <typename T2>
__device__ __forceinline__ T2 twiddle(const T2 *tw, int e, int sign) {
  T2 t = tw[e];
  if (sign > 0) t.y = -t.y;
  return t;
}

// In-register DFT of R points with exponent sign `sign` (-1 forward).
template <typename T2, int R>
struct SmallDft {
  __device__ __forceinline__ static void run(T2 *a, int sign, const T2 *tw, int L) {
    T2 y[R];
    const int step = L / R;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      T2 acc = a[0];
#pragma unroll
      for (int m = 1; m < R; ++m) acc = cadd(acc, cmul(a[m], twiddle(tw, ((m * q) % R) * step, sign)));
      y[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < R; ++q) a[q] = y[q];
  }
};

template <typename T2>
struct SmallDft<T2, 2> {
  __device__ __forceinline__ static void run(T2 *a, int, const T2 *, int) {
    const T2 t = a[1];
    a[1] = csub(a[0], t);
    a[0] = cadd(a[0], t);
  }
};

template <typename T2>
struct SmallDft<T2, 3> {
  __device__ __forceinline__ static void run(T2 *a, int sign, const T2 *, int) {
    using T = decltype(a[0].x);
    const T c = T(-0.5);
    const T s = T(0.86602540378443864676372317075294);  // sin(2 pi / 3)
    const T2 t1 = cadd(a[1], a[2]);
    const T2 t2 = csub(a[1], a[2]);
    T2 m;
    m.x = a[0].x + c * t1.x;
    m.y = a[0].y + c * t1.y;
    T2 r = cmul_isign(t2, sign);  // i*sign*(a1 - a2)
    r.x *= s;
    r.y *= s;
    a[0] = cadd(a[0], t1);
    a[1] = cadd(m, r);
    a[2] = csub(m, r);
  }
};

template <typename T2>
struct SmallDft<T2, 4> {
  __device__ __forceinline__ static void run(T2 *a, int sign, const T2 *, int) {
    const T2 t0 = cadd(a[0], a[2]);
    const T2 t1 = csub(a[0], a[2]);
    const T2 t2 = cadd(a[1], a[3]);
    const T2 t3 = cmul_isign(csub(a[1], a[3]), sign);
    a[0] = cadd(t0, t2);
    a[2] = csub(t0, t2);
    a[1] = cadd(t1, t3);
    a[3] = csub(t1, t3);
  }
};

template <typename T2>
struct SmallDft<T2, 8> {
  __device__ __forceinline__ static void run(T2 *a, int sign, const T2 *tw, int L) {
    using T = decltype(a[0].x);
    T2 e[4] = {a[0], a[2], a[4], a[6]};
    T2 o[4] = {a[1], a[3], a[5], a[7]};
    SmallDft<T2, 4>::run(e, sign, tw, L);
    SmallDft<T2, 4>::run(o, sign, tw, L);
    const T r = T(0.70710678118654752440084436210485);
    // W^1 = r (1 + i sign), W^2 = i sign, W^3 = r (-1 + i sign)
    T2 w1o, w2o, w3o;
    {
      const T2 t = cmul_isign(o[1], sign);
      w1o.x = r * (o[1].x + t.x);
      w1o.y = r * (o[1].y + t.y);
    }
    w2o = cmul_isign(o[2], sign);
    {
      const T2 t = cmul_isign(o[3], sign);
      w3o.x = r * (t.x - o[3].x);
      w3o.y = r * (t.y - o[3].y);
    }
    a[0] = cadd(e[0], o[0]);
    a[4] = csub(e[0], o[0]);
    a[1] = cadd(e[1], w1o);
    a[5] = csub(e[1], w1o);
    a[2] = cadd(e[2], w2o);
    a[6] = csub(e[2], w2o);
    a[3] = cadd(e[3], w3o);
    a[7] = csub(e[3], w3o);
  }
};

// One Stockham stage of radix R over P rows. Ns = product of earlier radices.
// POW2: L, R and Ns are powers of two and the index arithmetic uses shifts
// (lg_* are their base-2 logarithms); otherwise it divides.
template <typename T2, int R, int MAXE, int SIGN, bool POW2>
__device__ __forceinline__ void fft_stage(T2 *s, int LS, int P, int L, int Ns, const T2 *tw, int lg_nbf, int lg_ns) {
  constexpr int NB = MAXE / R;
  const int nbf = L / R;
  const int total = P * nbf;
  const int twstep = L / (Ns * R);
  T2 v[NB][R];
#pragma unroll
  for (int e = 0; e < NB; ++e) {
    const int b = threadIdx.x + e * blockDim.x;
    if (b < total) {
      int pp, j, k;
      if (POW2) {
        pp = b >> lg_nbf;
        j = b & (nbf - 1);
        k = j & (Ns - 1);
      } else {
        pp = b / nbf;
        j = b - pp * nbf;
        k = j % Ns;
      }
      const T2 *row = s + pp * LS;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        T2 x = row[j + q * nbf];
        if (q > 0 && k > 0) x = cmul(x, twiddle(tw, q * k * twstep, SIGN));
        v[e][q] = x;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int e = 0; e < NB; ++e) {
    const int b = threadIdx.x + e * blockDim.x;
    if (b < total) {
      SmallDft<T2, R>::run(v[e], SIGN, tw, L);
      int pp, j, k, out0;
      if (POW2) {
        pp = b >> lg_nbf;
        j = b & (nbf - 1);
        k = j & (Ns - 1);
        out0 = ((j >> lg_ns) << (lg_ns + __ffs(R) - 1)) + k;
      } else {
        pp = b / nbf;
        j = b - pp * nbf;
        k = j % Ns;
        out0 = (j / Ns) * Ns * R + k;
      }
      T2 *row = s + pp * LS;
#pragma unroll
      for (int q = 0; q < R; ++q) row[out0 + q * Ns] = v[e][q];
    }
  }
  __syncthreads();
}

// Direct O(L^2) DFT of every row (lengths with a large prime factor).
template <typename T2, int MAXE>
__device__ void dft_direct(T2 *s, int LS, int P, int L, int sign, const T2 *tw) {
  T2 y[MAXE];
  const int total = P * L;
#pragma unroll
  for (int e = 0; e < MAXE; ++e) {
    const int o = threadIdx.x + e * blockDim.x;
    if (o < total) {
      const int pp = o / L, q = o - pp * L;
      const T2 *row = s + pp * LS;
      T2 acc = row[0];
      long ex = 0;
      for (int m = 1; m < L; ++m) {
        ex += q;
        if (ex >= L) ex -= L;
        acc = cadd(acc, cmul(row[m], twiddle(tw, (int)ex, sign)));
      }
      y[e] = acc;
    }
  }
  __syncthreads();
#pragma unroll
  for (int e = 0; e < MAXE; ++e) {
    const int o = threadIdx.x + e * blockDim.x;
    if (o < total) {
      const int pp = o / L, q = o - pp * L;
      s[pp * LS + q] = y[e];
    }
  }
  __syncthreads();
}

struct FftFactors {
  int n;
  int f[16];
};

template <typename T2, int MAXE, int SIGN, bool POW2>
__device__ void fft_rows_t(T2 *s, int LS, int P, int L, const FftFactors &fac, const T2 *tw) {
  int Ns = 1, lg_ns = 0;
  for (int q = 0; q < fac.n; ++q) {
    const int R = fac.f[q];
    const int lg_nbf = POW2 ? (__ffs(L / R) - 1) : 0;
    switch (R) {
      case 2: fft_stage<T2, 2, MAXE, SIGN, POW2>(s, LS, P, L, Ns, tw, lg_nbf, lg_ns); break;
      case 4: fft_stage<T2, 4, MAXE, SIGN, POW2>(s, LS, P, L, Ns, tw, lg_nbf, lg_ns); break;
      case 8: fft_stage<T2, 8, MAXE, SIGN, POW2>(s, LS, P, L, Ns, tw, lg_nbf, lg_ns); break;
      case 3: if (!POW2) fft_stage<T2, 3, MAXE, SIGN, false>(s, LS, P, L, Ns, tw, 0, 0); break;
      case 5: if (!POW2) fft_stage<T2, 5, MAXE, SIGN, false>(s, LS, P, L, Ns, tw, 0, 0); break;
      case 7: if (!POW2) fft_stage<T2, 7, MAXE, SIGN, false>(s, LS, P, L, Ns, tw, 0, 0); break;
      case 11: if (!POW2) fft_stage<T2, 11, MAXE, SIGN, false>(s, LS, P, L, Ns, tw, 0, 0); break;
      case 13: if (!POW2) fft_stage<T2, 13, MAXE, SIGN, false>(s, LS, P, L, Ns, tw, 0, 0); break;
      default: if (!POW2) dft_direct<T2, MAXE>(s, LS, P, L, SIGN, tw); break;
    }
    Ns *= R;
    if (POW2) lg_ns += __ffs(R) - 1;
  }
}

// All rows of the CTA; `pow2` (uniform) selects the shift-indexed stages.
template <typename T2, int MAXE, int SIGN>
__device__ __forceinline__ void fft_rows(T2 *s, int LS, int P, int L, const FftFactors &fac, const T2 *tw, bool pow2) {
  if (pow2)
    fft_rows_t<T2, MAXE, SIGN, true>(s, LS, P, L, fac, tw);
  else
    fft_rows_t<T2, MAXE, SIGN, false>(s, LS, P, L, fac, tw);
}

}  // namespace mifgpu
