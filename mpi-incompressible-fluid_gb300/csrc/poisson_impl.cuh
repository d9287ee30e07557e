// Spectral Poisson solve on the owner block of phi (sm_103a).
//
// Restates solve_pressure_equation (src/PressureEquation.cpp:65-264) for one
// GPU: the same separable sequence — forward transforms along x, y, z, the
// product with 1/(lambda_x + lambda_y + lambda_z) (zero mode set to 0), inverse
// transforms along z, y, x with the reference's normalisations — but without
// the pencil transposes (deps/2Decomp_C/Transpose*.cpp): every sweep reads its
// lines in place with strided, coalesced tile loads, so the data never moves.
//
// Per axis the 1-D transform is the one FFTW computes in the reference
// (src/PressureSolverStructures.cpp:19-41): REDFT00 (DCT-I, unnormalised) on a
// Neumann axis, R2HC / HC2R on a periodic axis. Two real lines share one
// complex FFT: z = a + i b.
//   DCT-I, n points: FFT of length L = 2(n-1) of the even extension;
//                    Re/Im of the result are the two DCTs (real, even spectra).
//   R2HC,  n points: FFT of length n, then A_k = (Z_k + conj Z_{n-k})/2,
//                    B_k = (Z_k - conj Z_{n-k})/(2i), stored in FFTW's
//                    half-complex order r_0..r_{n/2}, i_{(n+1)/2-1}..i_1.
//   HC2R:            rebuild Z_k = A_k + i B_k from the two half-complex lines,
//                    inverse FFT, a = Re z, b = Im z.
// The z sweep fuses forward transform, eigenvalue product (in double) and
// inverse transform, so the spectrum along z never leaves shared memory.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

#include "fft.cuh"
#include "poisson.cuh"

namespace mifgpu {

namespace {

constexpr int kThreads = 256;

template <typename T>
struct MaxE;
template <>
struct MaxE<float> {
  static constexpr int v = 32;
};
template <>
struct MaxE<double> {
  static constexpr int v = 16;
};

enum { kModeForward = 0, kModeInverse = 1, kModeFwdEigInv = 2 };

template <typename T>
struct LineArgs {
  T *data;
  long se, sa, sb, base;  // element stride, strides of the two other axes, owner-block origin
  int na, nb;             // owner points along the two other axes (a varies fastest)
  int n, L, kind;         // points per line, complex FFT length, 0 DCT-I / 1 real DFT
  FftFactors fac;
  const typename Vec2<T>::type *tw;
  int P;          // line pairs per CTA
  int line_fast;  // 1: consecutive threads take consecutive lines (strided axes)
  double scale;   // output multiplier (inverse normalisation), 1 otherwise
  // kModeFwdEigInv only: eigenvalues of axes a, b and of the line axis
  const double *lam_a, *lam_b, *lam_n;
};

template <typename T>
__device__ __forceinline__ long line_offset(const LineArgs<T> &a, long gl) {
  const long qa = gl % a.na, qb = gl / a.na;
  return a.base + qa * a.sa + qb * a.sb;
}

// Global -> shared: line l of the CTA is component (l & 1) of row (l >> 1).
template <typename T, typename T2>
__device__ void load_lines(T2 *s, int LS, const LineArgs<T> &a, long line0, long total) {
  const int nl = 2 * a.P;
  const int cnt = nl * a.n;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    int l, m;
    if (a.line_fast) {
      m = e / nl;
      l = e - m * nl;
    } else {
      l = e / a.n;
      m = e - l * a.n;
    }
    const long gl = line0 + l;
    T v = T(0);
    if (gl < total) v = a.data[line_offset(a, gl) + (long)m * a.se];
    T *row = reinterpret_cast<T *>(s + (l >> 1) * LS);
    row[2 * m + (l & 1)] = v;
    if (a.kind == 0 && m > 0 && m < a.n - 1) row[2 * (a.L - m) + (l & 1)] = v;
  }
  __syncthreads();
}

template <typename T, typename T2>
__device__ void store_lines(const T2 *s, int LS, const LineArgs<T> &a, long line0, long total, T scale) {
  const int nl = 2 * a.P;
  const int cnt = nl * a.n;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    int l, m;
    if (a.line_fast) {
      m = e / nl;
      l = e - m * nl;
    } else {
      l = e / a.n;
      m = e - l * a.n;
    }
    const long gl = line0 + l;
    if (gl < total) {
      const T *row = reinterpret_cast<const T *>(s + (l >> 1) * LS);
      a.data[line_offset(a, gl) + (long)m * a.se] = row[2 * m + (l & 1)] * scale;
    }
  }
}

// Z (after a forward FFT of a + i b) -> the two half-complex spectra, stored
// as row[m] = (a_hc[m], b_hc[m]).
template <typename T2>
__device__ void split_halfcomplex(T2 *s, int LS, int P, int n) {
  using T = decltype(s[0].x);
  const int half = (n + 1) / 2;  // k in [1, half)
  const int cnt = P * (half - 1);
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int pp = e / (half - 1);
    const int k = 1 + e - pp * (half - 1);
    T2 *row = s + pp * LS;
    const T2 zk = row[k], zm = row[n - k];
    const T h = T(0.5);
    T2 lo, hi;
    lo.x = (zk.x + zm.x) * h;   // Re A_k
    lo.y = (zk.y + zm.y) * h;   // Re B_k
    hi.x = (zk.y - zm.y) * h;   // Im A_k
    hi.y = -(zk.x - zm.x) * h;  // Im B_k
    row[k] = lo;
    row[n - k] = hi;
  }
  __syncthreads();
}

// Two half-complex spectra row[m] = (a_hc[m], b_hc[m]) -> Z_k = A_k + i B_k.
template <typename T2>
__device__ void merge_halfcomplex(T2 *s, int LS, int P, int n) {
  const int half = (n + 1) / 2;
  const int cnt = P * (half - 1);
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int pp = e / (half - 1);
    const int k = 1 + e - pp * (half - 1);
    T2 *row = s + pp * LS;
    const T2 hk = row[k], hm = row[n - k];
    T2 zk, zm;
    zk.x = hk.x - hm.y;
    zk.y = hm.x + hk.y;
    zm.x = hk.x + hm.y;
    zm.y = hk.y - hm.x;
    row[k] = zk;
    row[n - k] = zm;
  }
  __syncthreads();
}

// Spectrum * 1/(lambda_a + lambda_b + lambda_n) in double, mode (0,0,0) := 0
// (src/PressureSolverStructures.cpp:52-69, src/PressureEquation.cpp:157-163).
template <typename T, typename T2>
__device__ void apply_eigenvalues(T2 *s, int LS, const LineArgs<T> &a, long line0, long total) {
  const int cnt = a.P * a.n;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int pp = e / a.n;
    const int m = e - pp * a.n;
    T2 *row = s + pp * LS;
    T2 v = row[m];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const long gl = line0 + 2 * pp + c;
      if (gl >= total) continue;
      const long qa = gl % a.na, qb = gl / a.na;
      const double lsum = a.lam_a[qa] + a.lam_b[qb] + a.lam_n[m];
      T &val = c == 0 ? v.x : v.y;
      if (qa == 0 && qb == 0 && m == 0)
        val = T(0);
      else
        val = T((double)val * (1.0 / lsum));
    }
    row[m] = v;
    if (a.kind == 0 && m > 0 && m < a.n - 1) row[a.L - m] = v;
  }
  __syncthreads();
}

template <typename T, int MODE>
__global__ void __launch_bounds__(kThreads) line_kernel(LineArgs<T> a) {
  using T2 = typename Vec2<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2 *s = reinterpret_cast<T2 *>(smem_raw);
  constexpr int MAXE = MaxE<T>::v;
  const int LS = a.L + 1;
  const long total = (long)a.na * a.nb;
  const long line0 = (long)blockIdx.x * 2 * a.P;

  load_lines(s, LS, a, line0, total);
  if (a.kind == 1 && MODE == kModeInverse) merge_halfcomplex(s, LS, a.P, a.n);
  const int sign0 = (a.kind == 1 && MODE == kModeInverse) ? +1 : -1;
  fft_rows<T2, MAXE>(s, LS, a.P, a.L, a.fac, sign0, a.tw);
  if (MODE == kModeFwdEigInv) {
    if (a.kind == 1) split_halfcomplex(s, LS, a.P, a.n);
    apply_eigenvalues(s, LS, a, line0, total);
    if (a.kind == 1) merge_halfcomplex(s, LS, a.P, a.n);
    fft_rows<T2, MAXE>(s, LS, a.P, a.L, a.fac, a.kind == 1 ? +1 : -1, a.tw);
  } else if (MODE == kModeForward && a.kind == 1) {
    split_halfcomplex(s, LS, a.P, a.n);
  }
  store_lines(s, LS, a, line0, total, T(a.scale));
}

int smallest_radix(int L) {
  static const int radices[] = {8, 4, 2, 3, 5, 7, 11, 13};
  for (int r : radices)
    if (L % r == 0) return r;
  return 0;
}

}  // namespace

// ---- host side ----

template <typename T>
int AxisPlan<T>::build(int kind_, int n_, double h, int line_count, bool line_fast_, std::string &err) {
  kind = kind_;
  n = n_;
  line_fast = line_fast_;
  if (n < 2) {
    err = "a Poisson axis needs at least 2 points";
    return -1;
  }
  L = kind == 0 ? 2 * (n - 1) : n;
  // Factorisation: radix 8 first, then 4, 2, 3, 5, 7, 11, 13; anything else
  // is one direct DFT of the whole length.
  nfac = 0;
  int rem = L;
  int cap = MaxE<T>::v;  // complex values one thread can hold per stage
  while (rem > 1) {
    const int r = smallest_radix(rem);
    if (r == 0) {
      nfac = 0;
      fac[nfac++] = L;
      cap = MaxE<T>::v;
      rem = 1;
      break;
    }
    fac[nfac++] = r;
    rem /= r;
    cap = std::min(cap, r * (MaxE<T>::v / r));
  }
  if (nfac == 1 && fac[0] == L && smallest_radix(L) == 0) cap = MaxE<T>::v;
  const long capacity = (long)kThreads * cap;
  if (L > capacity) {
    err = "Poisson line length " + std::to_string(n) + " exceeds the shared-memory FFT capacity";
    return -1;
  }
  P = (int)(capacity / L);
  const long max_pairs = (line_count + 1) / 2;
  if (P > max_pairs) P = (int)std::max<long>(1, max_pairs);
  const size_t row_bytes = sizeof(typename Vec2<T>::type) * (size_t)(L + 1);
  const size_t smem_cap = 96 * 1024;
  while (P > 1 && row_bytes * P > smem_cap) --P;
  smem = row_bytes * P;

  // Twiddles exp(-2 pi i e / L) in long double, rounded once.
  std::vector<typename Vec2<T>::type> hw(L);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int e = 0; e < L; ++e) {
    const long double ang = two_pi * (long double)e / (long double)L;
    hw[e].x = (T)cosl(ang);
    hw[e].y = (T)(-sinl(ang));
  }
  if (cudaMalloc(&tw, sizeof(hw[0]) * L) != cudaSuccess) {
    err = "cudaMalloc twiddles failed";
    return -2;
  }
  cudaMemcpy(tw, hw.data(), sizeof(hw[0]) * L, cudaMemcpyHostToDevice);

  // Eigenvalues of the discrete Laplacian along this axis, exactly as
  // src/PressureSolverStructures.cpp:5-11 computes them (double, host libm).
  std::vector<double> lam(n);
  for (int i = 0; i < n; ++i) {
    const size_t index = (size_t)i, N = (size_t)n;
    lam[i] = kind == 1 ? 2.0 * (std::cos(2.0 * M_PI * index / N) - 1.0) / (h * h)
                       : 2.0 * (std::cos(M_PI * index / (N - 1)) - 1.0) / (h * h);
  }
  if (cudaMalloc(&lam_dev, sizeof(double) * n) != cudaSuccess) {
    err = "cudaMalloc eigenvalues failed";
    return -2;
  }
  cudaMemcpy(lam_dev, lam.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
  return 0;
}

template <typename T>
void AxisPlan<T>::release() {
  if (tw) cudaFree(tw);
  if (lam_dev) cudaFree(lam_dev);
  tw = nullptr;
  lam_dev = nullptr;
}

template <typename T>
int PoissonSolver<T>::init(const Geometry &g, std::string &err) {
  geo = g;
  const int lines[3] = {g.np[1] * g.np[2], g.np[0] * g.np[2], g.np[0] * g.np[1]};
  size_t smem_max = 0;
  for (int d = 0; d < 3; ++d) {
    const int rc = axis[d].build(g.periodic[d] ? 1 : 0, g.np[d], g.h[d], lines[d], d != 0, err);
    if (rc) return rc;
    smem_max = std::max(smem_max, axis[d].smem);
  }
  // The limit is a property of the kernel function, shared by all three axes.
  for (int mode = 0; mode < 3; ++mode) {
    const void *fn = mode == 0   ? (const void *)line_kernel<T, kModeForward>
                     : mode == 1 ? (const void *)line_kernel<T, kModeInverse>
                                 : (const void *)line_kernel<T, kModeFwdEigInv>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max) != cudaSuccess) {
      err = "cudaFuncSetAttribute(MaxDynamicSharedMemorySize) failed";
      return -2;
    }
  }
  return 0;
}

template <typename T>
void PoissonSolver<T>::release() {
  for (auto &a : axis) a.release();
}

template <typename T>
static LineArgs<T> make_args(const Geometry &g, const AxisPlan<T> &ax, int d, T *phi) {
  LineArgs<T> a{};
  a.data = phi;
  const long stride[3] = {1, g.sy(), g.sz()};
  const int oa = d == 0 ? 1 : 0, ob = d == 2 ? 1 : 2;
  a.se = stride[d];
  a.sa = stride[oa];
  a.sb = stride[ob];
  a.na = g.np[oa];
  a.nb = g.np[ob];
  a.base = g.idx(g.own_lo[0], g.own_lo[1], g.own_lo[2]);
  a.n = ax.n;
  a.L = ax.L;
  a.kind = ax.kind;
  a.fac.n = ax.nfac;
  for (int q = 0; q < ax.nfac; ++q) a.fac.f[q] = ax.fac[q];
  a.tw = ax.tw;
  a.P = ax.P;
  a.line_fast = ax.line_fast ? 1 : 0;
  a.scale = 1.0;
  return a;
}

template <typename T>
int PoissonSolver<T>::solve(T *phi, cudaStream_t stream, long long *launches, const std::function<void(int)> &mark) {
  const Geometry &g = geo;
  // Inverse normalisations, src/PressureEquation.cpp:167,200,234:
  // (points - 1) * (periodic ? 1 : 2), applied as a product with the reciprocal.
  double norm[3];
  for (int d = 0; d < 3; ++d) norm[d] = 1.0 / ((double)(g.n_global[d] - 1) * (g.periodic[d] ? 1.0 : 2.0));
  auto launch = [&](int d, int mode, double scale) {
    const AxisPlan<T> &ax = axis[d];
    LineArgs<T> a = make_args(g, ax, d, phi);
    a.scale = scale;
    if (mode == kModeFwdEigInv) {
      a.lam_a = axis[0].lam_dev;  // the z sweep's other axes are x (fast) and y
      a.lam_b = axis[1].lam_dev;
      a.lam_n = axis[2].lam_dev;
    }
    const long total = (long)a.na * a.nb;
    const unsigned grid = (unsigned)((total + 2 * ax.P - 1) / (2 * ax.P));
    if (mode == kModeForward)
      line_kernel<T, kModeForward><<<grid, kThreads, ax.smem, stream>>>(a);
    else if (mode == kModeInverse)
      line_kernel<T, kModeInverse><<<grid, kThreads, ax.smem, stream>>>(a);
    else
      line_kernel<T, kModeFwdEigInv><<<grid, kThreads, ax.smem, stream>>>(a);
    if (launches) ++*launches;
  };
  const int seq_axis[5] = {0, 1, 2, 1, 0};
  const int seq_mode[5] = {kModeForward, kModeForward, kModeFwdEigInv, kModeInverse, kModeInverse};
  const double seq_scale[5] = {1.0, 1.0, norm[2], norm[1], norm[0]};
  for (int q = 0; q < 5; ++q) {
    if (mark) mark(q);
    launch(seq_axis[q], seq_mode[q], seq_scale[q]);
  }
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -2;
}

}  // namespace mifgpu
