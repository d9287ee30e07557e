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

#include <mutex>

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "fft.cuh"
#include "poisson.cuh"
#include "regfft.cuh"
#include "tma.cuh"

namespace mifgpu {

namespace {

constexpr int kThreads = 256;
// Threads of a register-path CTA (its line pairs: this over the FFT shape's
// second factor). The kernels take their thread count from the launch, up
// to kThreads. A CTA loads all its lines before its FFTs start, so its load
// and compute overlap only with other CTAs': at 128 threads six CTAs share an
// SM (the same 24 warps as three of 256). At 512^3 (32 x 16 shapes) the x, y
// and fused z sweeps took 0.89, 0.93 and 1.72 ms per step with 256 threads,
// 0.81, 0.85 and 1.66 with 128, 0.83, 0.91 and 1.86 with 64.
#ifndef MIFGPU_REG_THREADS
#define MIFGPU_REG_THREADS 128
#endif
constexpr int kRegThreads = MIFGPU_REG_THREADS;
static_assert(kRegThreads <= kThreads && (kRegThreads & (kRegThreads - 1)) == 0, "register-path CTA size");

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

constexpr int kMaxLines = 128;  // lines per CTA (2 P), a power of two

template <typename T>
struct LineArgs {
  T *data;
  long se, sa, sb, base;  // element stride, strides of the two other axes, owner-block origin
  int na, nb;             // owner points along the two other axes (a varies fastest)
  int n, L, kind;         // points per line, complex FFT length, 0 DCT-I / 1 real DFT /
                          // 2 DCT-I as a length n-1 transform (register path)
  FftFactors fac;
  int pow2;               // L is a power of two (shift-indexed FFT stages)
  const typename Vec2<T>::type *tw;
  const typename Vec2<T>::type *dsc;  // register path, kind 2: (sin, cos)(pi j / N)
  int P, lg_lines;        // line pairs per CTA; log2(2P)
  int line_fast;          // 1: consecutive threads take consecutive lines (strided axes)
  // Line enumeration along a: line g is (qa' = g % na_lines, qb = g / na_lines),
  // at owner index qa = qa' - lead, empty outside [0, na). With pair8 (register
  // path, strided axes with sa = 1), na_lines and lead make the two lines of
  // every pair adjacent and 8-byte aligned in memory, so a pair moves as one
  // 8-byte element; otherwise na_lines = na and lead = 0.
  int na_lines, lead, pair8;
  int vec16;              // x lines, register path, half-length DCT-I: 0, or the row pitch (floats)
                          // of the 16-byte staging (every line starts 16-byte aligned and its row
                          // holds the n points rounded up to 4)
  // Strided lines of the register path, half-length DCT-I, staged by TMA
  // (tma = 1): the CTA's lines in groups of four adjacent lines (na_lines and
  // lead make every group start 16-byte aligned), each group tma_chunks boxes
  // of 4 x tma_box elements of the kernel's tensor map at (x, line axis,
  // other axis) = (tma_x0 + qa', tma_m0 + chunk * tma_box, tma_b0 + qb), into
  // shared memory as [group][point][4] (a group every 4 tma_rows floats).
  int tma, tma_x0, tma_m0, tma_b0, tma_box, tma_chunks, tma_rows;
  int *err;               // set to 1 if a CTA gave up waiting for its TMA loads
  double scale;           // output multiplier (inverse normalisation), 1 otherwise
  // kModeFwdEigInv only: 1/(lambda_x + lambda_y + lambda_z) on the owner block,
  // z fastest, computed in double at set-up, zero mode 0.
  const T *eig;
};

// Per-CTA line table: global offset of each line's first element (-1 past the
// end) and its eigenvalue-table offset.
struct LineTable {
  long off[kMaxLines];
  long eoff[kMaxLines];
};

template <typename T>
__device__ void fill_line_table(LineTable &t, const LineArgs<T> &a, long line0, long total) {
  const int nl = 2 * a.P;
  for (int l = threadIdx.x; l < nl; l += blockDim.x) {
    const long gl = line0 + l;
    const long qa = gl % a.na_lines - a.lead, qb = gl / a.na_lines;
    if (gl < total && qa >= 0 && qa < a.na) {
      t.off[l] = a.base + qa * a.sa + qb * a.sb;
      t.eoff[l] = qa + (long)a.na * qb;  // (x, y) of a z line in the owner block
    } else {
      t.off[l] = -1;
      t.eoff[l] = 0;
    }
  }
  __syncthreads();
}

template <typename T>
__device__ __forceinline__ T line_value(const LineArgs<T> &a, long q) {
  return a.data[q];
}

template <typename T>
__device__ __forceinline__ void put(T *row, const LineArgs<T> &a, int l, int m, T v) {
  row[2 * m + (l & 1)] = v;
  if (a.kind == 0 && m > 0 && m < a.n - 1) row[2 * (a.L - m) + (l & 1)] = v;
}

// Global -> shared: line l of the CTA is component (l & 1) of row (l >> 1).
template <typename T, typename T2>
__device__ void load_lines(T2 *s, int LS, const LineArgs<T> &a, const LineTable &t) {
  const int nl = 2 * a.P;
  if (a.line_fast) {
    const int cnt = nl * a.n;
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const int m = e >> a.lg_lines, l = e & (nl - 1);
      const long off = t.off[l];
      const T v = off >= 0 ? line_value(a, off + (long)m * a.se) : T(0);
      put(reinterpret_cast<T *>(s + (l >> 1) * LS), a, l, m, v);
    }
  } else {
    for (int l = 0; l < nl; ++l) {
      const long off = t.off[l];
      T *row = reinterpret_cast<T *>(s + (l >> 1) * LS);
      for (int m = threadIdx.x; m < a.n; m += blockDim.x) put(row, a, l, m, off >= 0 ? line_value(a, off + m) : T(0));
    }
  }
  __syncthreads();
}

template <typename T, typename T2>
__device__ void store_lines(const T2 *s, int LS, const LineArgs<T> &a, const LineTable &t, T scale) {
  const int nl = 2 * a.P;
  if (a.line_fast) {
    const int cnt = nl * a.n;
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      const int m = e >> a.lg_lines, l = e & (nl - 1);
      const long off = t.off[l];
      if (off >= 0) {
        const T *row = reinterpret_cast<const T *>(s + (l >> 1) * LS);
        a.data[off + (long)m * a.se] = row[2 * m + (l & 1)] * scale;
      }
    }
  } else {
    for (int l = 0; l < nl; ++l) {
      const long off = t.off[l];
      if (off < 0) continue;
      const T *row = reinterpret_cast<const T *>(s + (l >> 1) * LS);
      for (int m = threadIdx.x; m < a.n; m += blockDim.x) a.data[off + m] = row[2 * m + (l & 1)] * scale;
    }
  }
}

// Z (after a forward FFT of a + i b) -> the two half-complex spectra, stored
// as row[m] = (a_hc[m], b_hc[m]).
template <typename T2>
__device__ void split_halfcomplex(T2 *s, int LS, int P, int n) {
  using T = decltype(s[0].x);
  const int half = (n + 1) / 2;  // k in [1, half)
  for (int pp = 0; pp < P; ++pp) {
    T2 *row = s + pp * LS;
    for (int k = 1 + threadIdx.x; k < half; k += blockDim.x) {
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
  }
  __syncthreads();
}

// Two half-complex spectra row[m] = (a_hc[m], b_hc[m]) -> Z_k = A_k + i B_k.
template <typename T2>
__device__ void merge_halfcomplex(T2 *s, int LS, int P, int n) {
  const int half = (n + 1) / 2;
  for (int pp = 0; pp < P; ++pp) {
    T2 *row = s + pp * LS;
    for (int k = 1 + threadIdx.x; k < half; k += blockDim.x) {
      const T2 hk = row[k], hm = row[n - k];
      T2 zk, zm;
      zk.x = hk.x - hm.y;
      zk.y = hm.x + hk.y;
      zm.x = hk.x + hm.y;
      zm.y = hk.y - hm.x;
      row[k] = zk;
      row[n - k] = zm;
    }
  }
  __syncthreads();
}

// Spectrum times the precomputed 1/(lambda_x + lambda_y + lambda_z)
// (src/PressureSolverStructures.cpp:52-69, src/PressureEquation.cpp:157-163).
template <typename T, typename T2>
__device__ void apply_eigenvalues(T2 *s, int LS, const LineArgs<T> &a, const LineTable &t) {
  for (int pp = 0; pp < a.P; ++pp) {
    T2 *row = s + pp * LS;
    const long ea = t.eoff[2 * pp] * a.n, eb = t.eoff[2 * pp + 1] * a.n;
    for (int m = threadIdx.x; m < a.n; m += blockDim.x) {
      T2 v = row[m];
      v.x = v.x * __ldg(a.eig + ea + m);
      v.y = v.y * __ldg(a.eig + eb + m);
      row[m] = v;
      if (a.kind == 0 && m > 0 && m < a.n - 1) row[a.L - m] = v;
    }
  }
  __syncthreads();
}

template <typename T, int MODE>
__global__ void __launch_bounds__(kThreads) line_kernel(LineArgs<T> a) {
  using T2 = typename Vec2<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ LineTable table;
  T2 *s = reinterpret_cast<T2 *>(smem_raw);
  constexpr int MAXE = MaxE<T>::v;
  const int LS = a.L + 1;
  const long total = (long)a.na_lines * a.nb;
  const long line0 = (long)blockIdx.x * 2 * a.P;
  const bool pow2 = a.pow2 != 0;

  fill_line_table(table, a, line0, total);
  load_lines(s, LS, a, table);
  if (MODE == kModeInverse && a.kind == 1) {
    merge_halfcomplex(s, LS, a.P, a.n);
    fft_rows<T2, MAXE, +1>(s, LS, a.P, a.L, a.fac, a.tw, pow2);
  } else {
    fft_rows<T2, MAXE, -1>(s, LS, a.P, a.L, a.fac, a.tw, pow2);
  }
  if (MODE == kModeFwdEigInv) {
    if (a.kind == 1) split_halfcomplex(s, LS, a.P, a.n);
    apply_eigenvalues(s, LS, a, table);
    if (a.kind == 1) {
      merge_halfcomplex(s, LS, a.P, a.n);
      fft_rows<T2, MAXE, +1>(s, LS, a.P, a.L, a.fac, a.tw, pow2);
    } else {
      fft_rows<T2, MAXE, -1>(s, LS, a.P, a.L, a.fac, a.tw, pow2);
    }
  } else if (MODE == kModeForward && a.kind == 1) {
    split_halfcomplex(s, LS, a.P, a.n);
  }
  store_lines(s, LS, a, table, T(a.scale));
}

// Inverse eigenvalue sums on the owner block, z fastest then x then y (the
// reference's z-pencil order), in double, as the reference tabulates them
// once (src/PressureSolverStructures.cpp:52-69). Zero mode: 0.
template <typename T>
__global__ void eigen_table_kernel(T *eig, const double *lx, const double *ly, const double *lz, int nx, int ny,
                                   int nz) {
  const long n = (long)nx * ny * nz;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (long)gridDim.x * blockDim.x) {
    const int k = (int)(id % nz), i = (int)((id / nz) % nx), j = (int)(id / ((long)nz * nx));
    eig[id] = (i == 0 && j == 0 && k == 0) ? T(0) : T(1.0 / (lx[i] + ly[j] + lz[k]));
  }
}

// ---- register-resident variant for power-of-two lengths (regfft.cuh) ----

// Asynchronous 4-byte global -> shared copy (no register staging, many in flight).
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::); }

// Element m of the first FFT's input for a real-DFT line pair: the plain
// pair (R2HC), or Z_k = A_k + i B_k rebuilt from two half-complex lines (HC2R).
template <typename T2, typename Src>
__device__ __forceinline__ T2 reg_input(const Src &src, int m, int L, bool hc2r) {
  if (!hc2r || m == 0 || 2 * m == L) return src(m);
  T2 z;
  if (2 * m < L) {
    const T2 hk = src(m), hm = src(L - m);
    z.x = hk.x - hm.y;
    z.y = hm.x + hk.y;
  } else {
    const T2 hk = src(L - m), hm = src(m);
    z.x = hk.x + hm.y;
    z.y = hk.y - hm.x;
  }
  return z;
}

// The z sweep's eigenvalue product for a periodic z axis, on the spectrum X
// of the pair (natural order in row), in place, by the N2 threads of the
// pair: eig_a A_m + i eig_b B_m with A = (X_m + conj X_-m)/2,
// B = (X_m - conj X_-m)/(2i), pairwise for (m, L-m), ea and eb the lines'
// rows of the 1/lambda table. (DCT-I lines are scaled by dct_half_output as
// it stores their spectra.)
template <typename T, int L>
__device__ __forceinline__ void reg_eig_row(typename Vec2<T>::type *row, int t, int stride, const T *ea,
                                            const T *eb) {
  using T2 = typename Vec2<T>::type;
  const T h = T(0.5);
  for (int m = t; 2 * m <= L; m += stride) {
    const int mn = m == 0 ? 0 : L - m;
    const T2 xm = row[m], xn = row[mn];
    T2 zm, zn;
    {
      const T ga = __ldg(ea + m) * h, gb = __ldg(eb + m) * h;
      zm.x = ga * (xm.x + xn.x) + gb * (xm.x - xn.x);
      zm.y = ga * (xm.y - xn.y) + gb * (xm.y + xn.y);
    }
    {
      const T ga = __ldg(ea + mn) * h, gb = __ldg(eb + mn) * h;
      zn.x = ga * (xn.x + xm.x) + gb * (xn.x - xm.x);
      zn.y = ga * (xn.y - xm.y) + gb * (xn.y + xm.y);
    }
    row[m] = zm;
    if (mn != m) row[mn] = zn;
  }
}

// DCT-I of N + 1 points (FFTW's REDFT00, unnormalised) from one length-N
// transform (the classic half-length algorithm): with s_j = x_j + x_{N-j} and
// d_j = x_j - x_{N-j}, the DFT Y of y_j = s_j / 2 - sin(pi j / N) d_j gives
//   X_{2k} = 2 Re Y_k,  X_{2k+1} = X_{2k-1} - 2 Im Y_k,
//   X_1 = sum_j d_j cos(pi j / N).
// Two lines travel as z = a + i b; their Y_k are split from Z_k and Z_{N-k}.

// Input element m = n1 N2 + t < N of z for the pair, and the pair's partial
// X_1. (sin, cos)(pi m / N) comes from the thread's own angle pi t / N
// (sct, from the table) and the compile-time angle pi n1 / N1 by the
// angle-addition formulas.
// The half-length DCT-I input arithmetic on the pair (packed FP32x2):
// s = xm + xn, d = xm - xn, v = s/2 - sin(pi m/N) d, x1 += cos(pi m/N) d, with
// (sin, cos)(pi m / N) from the thread's angle sct and the compile-time
// angle pi n1 / N1, each formed as a pair holding the value twice.
template <int N1>
__device__ __forceinline__ void dct_half_pre(float2 xm, float2 xn, int n1, float2 sct, float2 &v, float2 &x1) {
  static_assert(96 % N1 == 0, "pi n1 / N1 in the 192-entry table");
  const float cp = float(kCos192[n1 * (96 / N1)]), sp = float(kSin192[n1 * (96 / N1)]);
  const float2 sxx = make_float2(sct.x, sct.x), syy = make_float2(sct.y, sct.y);
  const float2 nsn = __ffma2_rn(syy, make_float2(-sp, -sp), __fmul2_rn(sxx, make_float2(-cp, -cp)));  // -sin
  const float2 cs = __ffma2_rn(sxx, make_float2(-sp, -sp), __fmul2_rn(syy, make_float2(cp, cp)));    // cos
  const float2 sm = cadd(xm, xn), d = csub(xm, xn);
  v = __ffma2_rn(nsn, d, __fmul2_rn(make_float2(0.5f, 0.5f), sm));
  x1 = __ffma2_rn(cs, d, x1);
}

template <typename T, int N1>
__device__ __forceinline__ void dct_half_input(const typename Vec2<T>::type *row, int m, int n1, int N,
                                               typename Vec2<T>::type sct, typename Vec2<T>::type &v,
                                               typename Vec2<T>::type &x1) {
  dct_half_pre<N1>(row[m], row[N - m], n1, sct, v, x1);
}

// The same from the 16-byte staging of contiguous x lines: the pair's two
// lines a, b in consecutive staging rows.
template <typename T, int N1>
__device__ __forceinline__ void dct_half_input_staged(const T *la, const T *lb, int m, int n1, int N,
                                                      typename Vec2<T>::type sct, typename Vec2<T>::type &v,
                                                      typename Vec2<T>::type &x1) {
  dct_half_pre<N1>(make_float2(la[m], lb[m]), make_float2(la[N - m], lb[N - m]), n1, sct, v, x1);
}

// The same from the TMA staging of strided lines: point m of the pair at
// g[4 m] (the pair's two lines adjacent in a group of four).
template <typename T, int N1>
__device__ __forceinline__ void dct_half_input_tma(const T *g, int m, int n1, int N, typename Vec2<T>::type sct,
                                                   typename Vec2<T>::type &v, typename Vec2<T>::type &x1) {
  dct_half_pre<N1>(*reinterpret_cast<const float2 *>(g + 4 * m), *reinterpret_cast<const float2 *>(g + 4 * (N - m)),
                   n1, sct, v, x1);
}

// Z of the pair in registers (x[r*N2 + k2] = Z_k, k = t + N2 (r + R k2),
// from reg_fft_core without STORE) -> row[m] = X_m (m <= N) of both lines.
// Thread t takes k = c N2 + t for c < C = N1/2 (k < N/2); the mirror Z_{N-k}
// is register c' = N1-1-c of lane N2-t (lane 0 keeps its own, c' = N1-c).
// The running sum of the odd outputs is taken over contiguous blocks of C
// values per thread, through a copy of D in the row at a padded index
// (k + k / C) that makes the strided and blocked accesses bank-conflict
// free, and an exclusive scan of the block totals across the lanes.
template <typename T, int N1, int N2>
__device__ __forceinline__ void dct_half_output(const typename Vec2<T>::type (&x)[N1], typename Vec2<T>::type *row,
                                                int t, typename Vec2<T>::type x1, const T *ea,
                                                const T *eb) {
  using T2 = typename Vec2<T>::type;
  constexpr int N = N1 * N2, C = N1 / 2, R = N1 / N2;
  static_assert(N2 <= 32 && (N1 % 2) == 0 && R >= 1, "pair within one warp");
  auto pad = [](int k) { return k + k / C; };
  auto reg = [](int c) { return (c % R) * N2 + c / R; };  // register of Z_{c N2 + t}
#pragma unroll
  for (int o = N2 / 2; o > 0; o >>= 1) {
    x1.x += __shfl_xor_sync(0xffffffffu, x1.x, o, N2);
    x1.y += __shfl_xor_sync(0xffffffffu, x1.y, o, N2);
  }
  const int partner = (N2 - t) & (N2 - 1);
  const T2 zh = x[reg(C)];  // Z_{N/2} on lane 0
  // A: even outputs, kept, and the odd-output increments D_k (D_0 = 0),
  // straight to the padded scratch (the row is free: reg_fft_core ended with
  // a warp barrier after its last read)
  T2 ev[C], dd[C];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const T2 zk = x[reg(c)];
    const T2 send = x[reg(N1 - 1 - c)];
    T2 zn;
    zn.x = __shfl_sync(0xffffffffu, send.x, partner, N2);
    zn.y = __shfl_sync(0xffffffffu, send.y, partner, N2);
    if (t == 0) zn = c == 0 ? zk : x[reg(N1 - c)];
    ev[c] = cadd(zk, zn);
    const bool k0 = c == 0 && t == 0;
    T2 d;
    d.x = k0 ? T(0) : zn.y - zk.y;
    d.y = k0 ? T(0) : zk.x - zn.x;
    row[pad(c * N2 + t)] = d;
  }
  __syncwarp();
  // C: blocked running sums, then the block offsets across the lanes
  T2 run = {T(0), T(0)};
#pragma unroll
  for (int c = 0; c < C; ++c) {
    run = cadd(run, row[pad(t * C + c)]);
    dd[c] = run;
  }
  T2 incl = run;
#pragma unroll
  for (int o = 1; o < N2; o <<= 1) {
    const T ux = __shfl_up_sync(0xffffffffu, incl.x, o, N2);
    const T uy = __shfl_up_sync(0xffffffffu, incl.y, o, N2);
    if (t >= o) {
      incl.x += ux;
      incl.y += uy;
    }
  }
  T2 excl;
  excl.x = __shfl_up_sync(0xffffffffu, incl.x, 1, N2);
  excl.y = __shfl_up_sync(0xffffffffu, incl.y, 1, N2);
  if (t == 0) excl.x = excl.y = T(0);
  __syncwarp();
#pragma unroll
  for (int c = 0; c < C; ++c) row[pad(t * C + c)] = cadd(x1, cadd(excl, dd[c]));
  __syncwarp();
  // D: the odd outputs back in the strided order
#pragma unroll
  for (int c = 0; c < C; ++c) dd[c] = row[pad(c * N2 + t)];
  __syncwarp();
  // E: X in natural order, X_2k and X_2k+1 as one 16-byte store; with the
  // 1/lambda rows ea, eb (the z sweep's first pass) scaled on the way
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int k = c * N2 + t;
    float4 o = make_float4(ev[c].x, ev[c].y, dd[c].x, dd[c].y);
    if (ea) {
      o.x *= __ldg(ea + 2 * k);
      o.y *= __ldg(eb + 2 * k);
      o.z *= __ldg(ea + 2 * k + 1);
      o.w *= __ldg(eb + 2 * k + 1);
    }
    *reinterpret_cast<float4 *>(row + 2 * k) = o;
  }
  if (t == 0) {
    T2 e;
    e.x = T(2) * zh.x;
    e.y = T(2) * zh.y;
    if (ea) {
      e.x *= __ldg(ea + N);
      e.y *= __ldg(eb + N);
    }
    row[N] = e;
  }
  __syncwarp();
}

// Twiddles W_L^(t k1), k1 = 1..N1-1, for thread t of a pair, one table
// read each. (Forming them as products W^(4ta) W^(tb) of fewer reads raised
// the 80-register kernels' spills, the loads being hoisted together.)
template <typename T, int N1, int L>
__device__ __forceinline__ void reg_twiddle_mul(typename Vec2<T>::type (&x)[N1], int t,
                                                const typename Vec2<T>::type *tw) {
#pragma unroll
  for (int k1 = 1; k1 < N1; ++k1) x[k1] = cmul(x[k1], __ldg(tw + t * k1));  // t k1 < N2 N1 = L
}

// One length-L forward FFT (exponent sign -1) of the pair owned by this
// thread group, in two register passes; x holds the thread's inputs
// x[n1] = z[n1*N2 + t]. With STORE the result X[k] lands in row[k],
// conjugated when conj_out is set (a sign +1 transform is
// conj(FFT(conj(z))): callers conjugate the input and set conj_out, so only
// one copy of this code exists per kernel); without STORE it stays in
// registers, x[r*N2 + k2] = X[t + r*N2 + N1*k2]. Every access is to the
// pair's own row, and a pair's N2 threads are lanes of one warp, so the
// phases are ordered by warp barriers.
template <typename T, int N1, int N2, bool STORE = true>
__device__ __forceinline__ void reg_fft_core(typename Vec2<T>::type (&x)[N1], typename Vec2<T>::type *row, int t,
                                             const typename Vec2<T>::type *tw, bool conj_out,
                                             bool cta_first = false) {
  using T2 = typename Vec2<T>::type;
  constexpr int L = N1 * N2;
  RegDft<T2, N1, -1>::run(x);
  reg_twiddle_mul<T, N1, L>(x, t, tw);
  // every thread of the pair has read its inputs from the row (with
  // cta_first the inputs came from a CTA-wide staging the rows overlap)
  if (cta_first)
    __syncthreads();
  else
    __syncwarp();
#pragma unroll
  for (int k1 = 0; k1 < N1; ++k1) row[k1 * (N2 + 1) + t] = x[k1];
  __syncwarp();
  constexpr int R = N1 / N2;  // columns per thread
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int k1 = t + r * N2;
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) x[r * N2 + n2] = row[k1 * (N2 + 1) + n2];
    RegDft<T2, N2, -1>::run(x + r * N2);
  }
  __syncwarp();
  if constexpr (STORE) {
    const T sy = conj_out ? T(-1) : T(1);
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) {
        T2 v = x[r * N2 + k2];
        v.y *= sy;
        row[t + r * N2 + N1 * k2] = v;
      }
    __syncwarp();
  }
}

// The register budget of three kThreads-thread CTAs per SM (at most 80
// registers; with kRegThreads = 128, six CTAs of half the size). The fused
// z sweep spills ~200 bytes at that bound but still ran 2.5% faster on GB300
// than with 128 registers. The 48-point shapes keep the budget of two (96
// registers of data; their rows allow no more CTAs anyway).
template <int N1, int MODE>
struct RegMinBlocks {
  static constexpr int v = N1 >= 48 ? 2 : 3;
};

template <typename T, int N1, int N2, int MODE, int KIND>
__global__ void __launch_bounds__(kThreads, RegMinBlocks<N1, MODE>::v)
    line_kernel_reg(LineArgs<T> a, const __grid_constant__ CUtensorMap tmap) {
  static_assert(sizeof(T) == 4, "the register path stages 4-byte elements");
  static_assert(KIND == 1 || KIND == 2, "real DFT or half-length DCT-I");
  using T2 = typename Vec2<T>::type;
  constexpr int L = N1 * N2;
  constexpr int ROW = RegShape<N1, N2>::ROW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ LineTable table;
  __shared__ uint64_t tbar;
  T2 *s = reinterpret_cast<T2 *>(smem_raw);
  // the TMA staging starts 128-byte aligned inside the rows (their bytes
  // exceed the staging's by more than 128)
  T *const stg = reinterpret_cast<T *>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
  const bool tma = KIND == 2 && a.tma;
  const long total = (long)a.na_lines * a.nb;
  const long line0 = (long)blockIdx.x * 2 * a.P;
  const int pp = threadIdx.x / N2, t = threadIdx.x % N2;
  T2 *row = s + pp * ROW;
  const int n = a.n;
  const int nl = 2 * a.P;

  if (tma && threadIdx.x == 0) {
    mbar_init(&tbar, 1);
    mbar_init_fence();
  }
  fill_line_table(table, a, line0, total);  // (ends with a CTA barrier)
  // One 128-byte global segment per warp access: strided lines put 32
  // consecutive lines (consecutive addresses) on the lanes of a warp at one m,
  // x lines put a warp on one line. (Splitting a warp into two 16-line or
  // two-line halves makes the 4-byte shared-memory writes conflict free but
  // halves the segments, and ran slower.)
  if (tma) {
    // thread 0 loads the P / 2 groups of four lines; every thread waits
    if (threadIdx.x == 0) {
      const int ng = a.P / 2;
      mbar_expect_tx(&tbar, (unsigned)(ng * a.tma_rows * 4 * sizeof(T)));
      for (int q = 0; q < ng; ++q) {
        const long g0 = line0 + 4 * q;
        const int x = a.tma_x0 + (int)(g0 % a.na_lines), b = a.tma_b0 + (int)(g0 / a.na_lines);
        for (int c = 0; c < a.tma_chunks; ++c)
          tma_load_3d(stg + (q * a.tma_rows + c * a.tma_box) * 4, &tmap, x, a.tma_m0 + c * a.tma_box, b, &tbar);
      }
    }
  } else if (a.line_fast && a.pair8) {
    // pair p of the CTA is lines 2p, 2p+1, adjacent in memory from an even
    // address: one 8-byte copy per point (16 pairs of a warp span 128 bytes)
    const int p = threadIdx.x & (a.P - 1), ms = blockDim.x >> (a.lg_lines - 1);
    const long offa = table.off[2 * p], offb = table.off[2 * p + 1];
    T2 *dst = s + p * ROW;
    if (offa >= 0 && offb >= 0) {
      const T *src0 = a.data + offa;
      for (int m = threadIdx.x >> (a.lg_lines - 1); m < n; m += ms) cp_async8(dst + m, src0 + (long)m * a.se);
    } else {
      // a row edge: the valid line alone, the empty one zero
      T *da = reinterpret_cast<T *>(dst), *db = da + 1;
      for (int m = threadIdx.x >> (a.lg_lines - 1); m < n; m += ms) {
        if (offa >= 0) cp_async4(da + 2 * m, a.data + offa + (long)m * a.se); else da[2 * m] = T(0);
        if (offb >= 0) cp_async4(db + 2 * m, a.data + offb + (long)m * a.se); else db[2 * m] = T(0);
      }
    }
  } else if (a.line_fast) {
    const int l = threadIdx.x & (nl - 1);
    const long off = table.off[l];
    T *dst = reinterpret_cast<T *>(s + (l >> 1) * ROW) + (l & 1);
    const int ms = blockDim.x >> a.lg_lines;
    if (off >= 0) {
      const T *src0 = a.data + off;
      for (int m = threadIdx.x >> a.lg_lines; m < n; m += ms) cp_async4(dst + 2 * m, src0 + (long)m * a.se);
    } else {
      for (int m = threadIdx.x >> a.lg_lines; m < n; m += ms) dst[2 * m] = T(0);
    }
  } else if (KIND == 2 && MODE != kModeFwdEigInv && a.vec16) {
    // Contiguous, 16-byte aligned x lines: line l in its own staging row of
    // a.vec16 floats, 16-byte copies (the elements past n are read from the
    // row padding and never used).
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5, nv = (n + 3) >> 2;
    for (int l = threadIdx.x >> 5; l < nl; l += nw) {
      const long off = table.off[l];
      float4 *dst = reinterpret_cast<float4 *>(reinterpret_cast<T *>(smem_raw) + (long)l * a.vec16);
      if (off >= 0) {
        const float4 *src0 = reinterpret_cast<const float4 *>(a.data + off);
        for (int v = lane; v < nv; v += 32) cp_async16(dst + v, src0 + v);
      } else {
        for (int v = lane; v < nv; v += 32) dst[v] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
  } else {
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int l = threadIdx.x >> 5; l < nl; l += nw) {
      const long off = table.off[l];
      T *dst = reinterpret_cast<T *>(s + (l >> 1) * ROW) + (l & 1);
      if (off >= 0) {
        const T *src0 = a.data + off;
        for (int m = lane; m < n; m += 32) cp_async4(dst + 2 * m, src0 + m);
      } else {
        for (int m = lane; m < n; m += 32) dst[2 * m] = T(0);
      }
    }
  }
  if (MODE == kModeFwdEigInv) {
    // The CTA's 1/lambda rows (consecutive lines, z fastest: one contiguous
    // range) towards L2 while the lines load; the first pass reads them when
    // it stores its spectra.
    const long last = min(line0 + nl, total) - 1;
    const char *e0 = reinterpret_cast<const char *>(a.eig + table.eoff[0] * n);
    const char *e1 = reinterpret_cast<const char *>(a.eig + (table.eoff[last - line0] + 1) * n);
    if (table.eoff[last - line0] == table.eoff[0] + (last - line0))
      for (const char *q = e0 + 128 * threadIdx.x; q < e1; q += 128 * blockDim.x)
        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(q));
  }
  if (tma) {
    // a wait that gives up is recorded; the CTA still runs to its end
    if (!mbar_wait(&tbar, 0) && a.err) atomicExch(a.err, 1);
  } else {
    cp_async_wait_all();
    __syncthreads();
  }
  const T2 *src = row;
  // (the fused z sweep's lines are always strided: no x-line staging there)
  const bool staged = KIND == 2 && MODE != kModeFwdEigInv && !a.line_fast && a.vec16;
  const T *ea = nullptr, *eb = nullptr;
  if (MODE == kModeFwdEigInv) ea = a.eig + table.eoff[2 * pp] * n, eb = a.eig + table.eoff[2 * pp + 1] * n;
  constexpr int npass = MODE == kModeFwdEigInv ? 2 : 1;
#pragma unroll 1
  for (int pass = 0; pass < npass; ++pass) {
    // pass 0: forward, or HC2R for the inverse real DFT; pass 1: eigenvalue
    // product and the inverse transform of the z sweep
    const bool plus = KIND == 1 && (MODE == kModeInverse || pass == 1);
    if (pass == 1) {
      if (KIND != 2) {
        reg_eig_row<T, L>(row, t, N2, ea, eb);
        __syncwarp();
      }
    }
    T2 x[N1];
    T2 x1 = {T(0), T(0)};  // kind 2: the pair's partial X_1
    T2 sct = {T(0), T(1)};
    if (KIND == 2) sct = __ldg(a.dsc + t);
    // the first FFT's inputs, one unrolled loop per input layout (the layout
    // is uniform across the CTA, chosen once)
    auto gather = [&](auto input) {
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) {
        T2 v;
        input(n1 * N2 + t, n1, v);
        if (plus) v.y = -v.y;
        x[n1] = v;
      }
    };
    if constexpr (KIND == 2) {
      if (tma && pass == 0) {
        const T *g = stg + (pp >> 1) * a.tma_rows * 4 + (pp & 1) * 2;
        gather([&](int m, int n1, T2 &v) { dct_half_input_tma<T, N1>(g, m, n1, L, sct, v, x1); });
      } else if (staged && pass == 0) {
        const T *lab = reinterpret_cast<const T *>(smem_raw) + (long)2 * pp * a.vec16;
        gather([&](int m, int n1, T2 &v) { dct_half_input_staged<T, N1>(lab, lab + a.vec16, m, n1, L, sct, v, x1); });
      } else {
        gather([&](int m, int n1, T2 &v) { dct_half_input<T, N1>(row, m, n1, L, sct, v, x1); });
      }
    } else {
      gather([&](int m, int, T2 &v) {
        v = pass == 0 ? reg_input<T2>([&](int q) { return src[q]; }, m, L, MODE == kModeInverse) : row[m];
      });
    }
    if constexpr (KIND == 2) {
      reg_fft_core<T, N1, N2, false>(x, row, t, a.tw, false, (staged || tma) && pass == 0);
      const bool scale_eig = MODE == kModeFwdEigInv && pass == 0;
      dct_half_output<T, N1, N2>(x, row, t, x1, scale_eig ? ea : nullptr, scale_eig ? eb : nullptr);
    } else {
      reg_fft_core<T, N1, N2>(x, row, t, a.tw, plus);
    }
  }
  __syncthreads();  // the stores below read other pairs' rows
  // store: row[m] holds X[m]; the forward real DFT splits the pair into
  // FFTW's half-complex order on the way out.
  const T scale = T(a.scale);
  const bool split = MODE == kModeForward && KIND == 1;
  auto value = [&](const T2 *r, int m, int comp) -> T {
    if (!split) return (comp ? r[m].y : r[m].x) * scale;
    const T2 xm = r[m], xn = r[m == 0 ? 0 : L - m];
    const T h = T(0.5);
    if (2 * m <= L) return comp ? (xm.y + xn.y) * h : (xm.x + xn.x) * h;
    return comp ? (xm.x - xn.x) * h : (xn.y - xm.y) * h;
  };
  if (a.line_fast && a.pair8) {
    // one 8-byte store per point for a pair of adjacent lines
    const int p = threadIdx.x & (a.P - 1), ms = blockDim.x >> (a.lg_lines - 1);
    const long offa = table.off[2 * p], offb = table.off[2 * p + 1];
    const T2 *r = s + p * ROW;
    if (offa >= 0 && offb >= 0) {
      T2 *dst0 = reinterpret_cast<T2 *>(a.data + offa);
      const long se2 = a.se / 2;
      for (int m = threadIdx.x >> (a.lg_lines - 1); m < n; m += ms) {
        T2 o;
        o.x = value(r, m, 0);
        o.y = value(r, m, 1);
        dst0[(long)m * se2] = o;
      }
    } else {
      for (int m = threadIdx.x >> (a.lg_lines - 1); m < n; m += ms) {
        if (offa >= 0) a.data[offa + (long)m * a.se] = value(r, m, 0);
        if (offb >= 0) a.data[offb + (long)m * a.se] = value(r, m, 1);
      }
    }
  } else if (a.line_fast) {
    const int l = threadIdx.x & (nl - 1);
    const long off = table.off[l];
    if (off >= 0) {
      const T2 *r = s + (l >> 1) * ROW;
      T *dst0 = a.data + off;
      const int ms = blockDim.x >> a.lg_lines;
      for (int m = threadIdx.x >> a.lg_lines; m < n; m += ms) dst0[(long)m * a.se] = value(r, m, l & 1);
    }
  } else {
    // one warp per line pair: each lane reads a complex element once and
    // writes it to both lines
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int p2 = threadIdx.x >> 5; p2 < nl / 2; p2 += nw) {
      const long offa = table.off[2 * p2], offb = table.off[2 * p2 + 1];
      const T2 *r = s + p2 * ROW;
      T *da = a.data + offa, *db = a.data + offb;
      for (int m = lane; m < n; m += 32) {
        if (offa >= 0) da[m] = value(r, m, 0);
        if (offb >= 0) db[m] = value(r, m, 1);
      }
    }
  }
}

int smallest_radix(int L) {
  static const int radices[] = {8, 4, 2, 3, 5, 7, 11, 13};
  for (int r : radices)
    if (L % r == 0) return r;
  return 0;
}

}  // namespace

// ---- host side ----

// Kernel pointer of the register path for FFT shape (A, B), mode and kind.
// Instantiated explicitly for float, one shape per translation unit
// (poisson_reg_*.cu), so the shapes compile in parallel.
template <typename T, int A, int B>
const void *reg_kernel_ptr(int mode, int kind) {
  if (kind == 2)
    return mode == kModeForward   ? (const void *)line_kernel_reg<T, A, B, kModeForward, 2>
           : mode == kModeInverse ? (const void *)line_kernel_reg<T, A, B, kModeInverse, 2>
                                  : (const void *)line_kernel_reg<T, A, B, kModeFwdEigInv, 2>;
  if (kind != 1) return nullptr;  // a DCT-I axis always takes the half-length form (kind 2) here
  return mode == kModeForward   ? (const void *)line_kernel_reg<T, A, B, kModeForward, 1>
         : mode == kModeInverse ? (const void *)line_kernel_reg<T, A, B, kModeInverse, 1>
                                : (const void *)line_kernel_reg<T, A, B, kModeFwdEigInv, 1>;
}

#define MIFGPU_REG_SHAPES(X) X(8, 8) X(16, 8) X(16, 16) X(32, 16) X(32, 32) X(48, 8) X(48, 16)
#ifndef MIFGPU_REG_TU
#define MIFGPU_REG_EXTERN(A, B) extern template const void *reg_kernel_ptr<float, A, B>(int, int);
MIFGPU_REG_SHAPES(MIFGPU_REG_EXTERN)
#undef MIFGPU_REG_EXTERN
#endif

template <typename T>
struct RegKernels {
  static const void *get(int n1, int n2, int mode, int kind) {
    if constexpr (std::is_same<T, float>::value) {
#define MIFGPU_REG_GET(A, B) \
  if (n1 == A && n2 == B) return reg_kernel_ptr<T, A, B>(mode, kind);
      MIFGPU_REG_SHAPES(MIFGPU_REG_GET)
#undef MIFGPU_REG_GET
    }
    return nullptr;
  }
};

template <typename T>
static void launch_reg(int n1, int n2, int mode, unsigned grid, size_t smem, cudaStream_t stream, LineArgs<T> a,
                       const CUtensorMap &tmap) {
  const void *fn = RegKernels<T>::get(n1, n2, mode, a.kind);
  CUtensorMap map = tmap;
  void *args[] = {&a, &map};
  cudaLaunchKernel(fn, dim3(grid), dim3(a.P * (unsigned)n2), args, smem, stream);
}


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
  if (P > kMaxLines / 2) P = kMaxLines / 2;
  const size_t row_bytes = sizeof(typename Vec2<T>::type) * (size_t)(L + 1);
  const size_t smem_cap = 96 * 1024;
  while (P > 1 && row_bytes * P > smem_cap) --P;
  while (P & (P - 1)) --P;  // a power of two: line indices split with shifts
  lg_lines = 0;
  while ((1 << lg_lines) < 2 * P) ++lg_lines;
  pow2 = (L & (L - 1)) == 0;
  if (pow2)
    for (int q = 0; q < nfac; ++q)
      if (fac[q] & (fac[q] - 1)) pow2 = false;
  smem = row_bytes * P;
  // Register-resident path (regfft.cuh): float, a power-of-two transform in
  // [64, 1024]: the real DFT of a periodic line, or for a DCT-I line of
  // n = N + 1 points the length-N transform of the half-length algorithm.
  reg_n1 = reg_n2 = reg_L = 0;
  reg_half = false;
  const int cand = kind == 0 ? n - 1 : n;
  const bool pow2_cand = (cand & (cand - 1)) == 0 && cand >= 64 && cand <= 1024;
  if (std::is_same<T, float>::value && (pow2_cand || cand == 384 || cand == 768)) {
    reg_L = cand;
    reg_half = kind == 0;
    if (pow2_cand) {
      int lg = 0;
      while ((1 << lg) < reg_L) ++lg;
      reg_n1 = 1 << ((lg + 1) / 2);
    } else {
      reg_n1 = 48;  // 3 x 2^k: 48 x 8 or 48 x 16
    }
    reg_n2 = reg_L / reg_n1;
    reg_P = kRegThreads / reg_n2;
    reg_lg = 0;
    while ((1 << reg_lg) < 2 * reg_P) ++reg_lg;
    reg_smem = sizeof(typename Vec2<T>::type) * (size_t)reg_P * (size_t)(reg_n1 * (reg_n2 + 1) + 2);  // RegShape::ROW
  }

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
  reg_tw = tw;
  if (reg_n1 && reg_L != L) {
    std::vector<typename Vec2<T>::type> rw(reg_L), sc(reg_L);
    for (int e = 0; e < reg_L; ++e) {
      const long double ang = two_pi * (long double)e / (long double)reg_L;
      rw[e].x = (T)cosl(ang);
      rw[e].y = (T)(-sinl(ang));
      const long double half = ang / 2;  // pi e / N
      sc[e].x = (T)sinl(half);
      sc[e].y = (T)cosl(half);
    }
    if (cudaMalloc(&reg_tw, sizeof(rw[0]) * reg_L) != cudaSuccess ||
        cudaMalloc(&dsc, sizeof(sc[0]) * reg_L) != cudaSuccess) {
      err = "cudaMalloc of the half-length DCT tables failed";
      return -2;
    }
    cudaMemcpy(reg_tw, rw.data(), sizeof(rw[0]) * reg_L, cudaMemcpyHostToDevice);
    cudaMemcpy(dsc, sc.data(), sizeof(sc[0]) * reg_L, cudaMemcpyHostToDevice);
  }

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
  if (reg_tw && reg_tw != tw) cudaFree(reg_tw);
  if (dsc) cudaFree(dsc);
  if (tw) cudaFree(tw);
  if (lam_dev) cudaFree(lam_dev);
  tw = reg_tw = dsc = nullptr;
  lam_dev = nullptr;
}

// The dynamic shared-memory limit is an attribute of the kernel, shared by
// every solver of the process: raise it to what this solver needs, never lower
// it below what an earlier (still live) solver set.
inline cudaError_t raise_dynamic_smem(const void *fn, size_t bytes) {
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  cudaFuncAttributes fa{};
  cudaError_t e = cudaFuncGetAttributes(&fa, fn);
  if (e != cudaSuccess) return e;
  if ((size_t)fa.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
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
  // 1/(lambda_x + lambda_y + lambda_z) on the owner block, in double once.
  const size_t ne = (size_t)g.np[0] * g.np[1] * g.np[2];
  if (cudaMalloc(&eig, sizeof(T) * ne) != cudaSuccess) {
    err = "cudaMalloc of the eigenvalue table failed";
    return -2;
  }
  eigen_table_kernel<T><<<1024, 256>>>(eig, axis[0].lam_dev, axis[1].lam_dev, axis[2].lam_dev, g.np[0], g.np[1],
                                       g.np[2]);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    err = "eigenvalue table kernel failed";
    return -2;
  }
  for (int d = 0; d < 3; ++d) {
    if (!axis[d].reg_n1) continue;
    for (int mode = 0; mode < 3; ++mode) {
      const void *fn = RegKernels<T>::get(axis[d].reg_n1, axis[d].reg_n2, mode, axis[d].reg_half ? 2 : axis[d].kind);
      if (!fn || raise_dynamic_smem(fn, axis[d].reg_smem) != cudaSuccess) {
        err = "register-path kernel set-up failed";
        return -2;
      }
    }
  }
  // The limit is a property of the kernel function, shared by all three axes.
  for (int mode = 0; mode < 3; ++mode) {
    const void *fn = mode == 0   ? (const void *)line_kernel<T, kModeForward>
                     : mode == 1 ? (const void *)line_kernel<T, kModeInverse>
                                 : (const void *)line_kernel<T, kModeFwdEigInv>;
    if (raise_dynamic_smem(fn, smem_max) != cudaSuccess) {
      err = "cudaFuncSetAttribute(MaxDynamicSharedMemorySize) failed";
      return -2;
    }
  }
  return 0;
}

template <typename T>
void PoissonSolver<T>::release() {
  for (auto &a : axis) a.release();
  if (eig) cudaFree(eig);
  eig = nullptr;
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
  a.pow2 = ax.pow2 ? 1 : 0;
  a.tw = ax.tw;
  a.P = ax.P;
  a.lg_lines = ax.lg_lines;
  a.line_fast = ax.line_fast ? 1 : 0;
  a.na_lines = a.na;
  a.lead = 0;
  a.pair8 = 0;
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
    if (mode == kModeFwdEigInv) a.eig = eig;  // the z sweep's other axes are x (fast) and y
    if (ax.reg_n1 && a.line_fast && a.sa == 1 && a.se % 2 == 0 && a.sb % 2 == 0) {
      // strided lines along x-adjacent columns: enumerate them from an even
      // address (lead: the odd owner origin of a periodic x axis) in rows of
      // an even count, so every pair is one aligned 8-byte element
      a.lead = (int)(a.base % 2);
      a.na_lines = (a.na + a.lead + 1) / 2 * 2;
      a.pair8 = 1;
    }
    if (ax.reg_n1) {
      a.P = ax.reg_P;
      a.lg_lines = ax.reg_lg;
      a.L = ax.reg_L;
      a.tw = ax.reg_tw;
      a.dsc = ax.dsc;
      if (ax.reg_half) a.kind = 2;
      a.vec16 = 0;
      CUtensorMap tmap{};
      if (std::is_same<T, float>::value && a.kind == 2 && a.pair8 && d != 0 && a.P % 2 == 0) {
        // TMA staging of the strided y / z lines in groups of four: the
        // line axis in tma_chunks boxes of at most 256 points (a multiple of
        // 8, so every box lands 128-byte aligned), groups from a 16-byte
        // aligned x (lead: the owner origin's offset from it)
        const int chunks = (a.n + 255) / 256;
        const int box = ((a.n + chunks - 1) / chunks + 7) / 8 * 8;
        const int rows = chunks * box, lead = g.own_lo[0] % 4;
        const bool fits = (long)(a.P / 2) * rows * 4 * (long)sizeof(T) + 128 <= (long)ax.reg_smem;
        const long dims[3] = {g.PX, d == 1 ? g.PY : g.PZ, d == 1 ? g.PZ : g.PY};
        const long strides[2] = {(d == 1 ? g.sy() : g.sz()) * (long)sizeof(T),
                                 (d == 1 ? g.sz() : g.sy()) * (long)sizeof(T)};
        if (fits && box <= 256 && make_map_3d(&tmap, phi, (int)sizeof(T), dims, strides, 4, box)) {
          a.tma = 1;
          a.lead = lead;
          a.na_lines = (a.na + lead + 3) / 4 * 4;
          a.tma_x0 = g.own_lo[0] - lead;
          a.tma_m0 = g.own_lo[d];
          a.tma_b0 = g.own_lo[d == 1 ? 2 : 1];
          a.tma_box = box;
          a.tma_chunks = chunks;
          a.tma_rows = rows;
          a.err = err_flag;
        }
      }
      if (d == 0 && a.kind == 2) {
        // 16-byte staging of the x lines: every line start 16-byte aligned
        // (the strides are multiples of 8 elements), the rounded-up line
        // inside its padded row, and the staging inside the kernel's rows.
        // The pitch is a multiple of 4 with 2 x pitch = 16 mod 32 banks, so
        // the two pairs of a warp read disjoint banks.
        long pitch = (a.n + 3) / 4 * 4;
        while (pitch % 16 != 8) pitch += 4;
        const long nl = 2L * a.P;
        const bool aligned = a.base % 4 == 0 && a.sa % 4 == 0 && a.sb % 4 == 0;
        const bool in_row = (long)g.own_lo[0] + (a.n + 3) / 4 * 4 <= g.PX;
        if (aligned && in_row && nl * pitch * (long)sizeof(T) <= (long)ax.reg_smem) a.vec16 = (int)pitch;
      }
      const long total = (long)a.na_lines * a.nb;
      const unsigned grid = (unsigned)((total + 2 * a.P - 1) / (2 * a.P));
      launch_reg<T>(ax.reg_n1, ax.reg_n2, mode, grid, ax.reg_smem, stream, a, tmap);
      if (launches) ++*launches;
      return;
    }
    const long total = (long)a.na_lines * a.nb;
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
