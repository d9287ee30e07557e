// Point-wise kernels of the time step (sm_103a): the three RK stage updates
// with the fused momentum right-hand side, the boundary fill, the divergence,
// the projection, layout conversion and the double-precision reductions.
//
// All three velocity components of a stage are computed by one thread per
// point, so each launch streams the stage's inputs once. Expressions keep the
// reference's evaluation order (include/MomentumEquation.h:42-255,
// src/Timestep.cpp:10-54) so FP64 results stay within rounding of the CPU
// solver.
#pragma once

#include <type_traits>

#include <cmath>

#include "analytic.cuh"
#include "stencil.cuh"
#include "tma.cuh"

namespace mifgpu {

namespace {

template <typename T>
__device__ __forceinline__ T ld(const T *p, long q) {
  return __ldg(p + q);
}

// ---- stochastic rounding of FP32 state updates (mixed precision) ----
//
// A stage adds an increment of O(dt) to an O(1) velocity; rounded to the
// nearest float the increment loses a biased share of its bits every time,
// and with dt ~ h^2 that error grows with the number of stages (increments
// below half an ulp are lost entirely). The state updates of the float path
// therefore round stochastically, in the dithered form: uniform noise in
// [-1/2, 1/2) ulp of the state is added to the increment before the
// round-to-nearest addition, so the rounded sum equals the exact one in
// expectation and the rounding errors add up as a random walk. The draws come
// from a counter-based hash of the point, the stage and the step's time (ten
// bits per update), so a run is deterministic.
__device__ __forceinline__ unsigned sr_mix(unsigned x) {
  // lowbias32 integer hash (public domain)
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Per-launch salt from the step's time t_n (time slot 0) and a stage tag.
__device__ __forceinline__ unsigned sr_salt(const TimeRef &tr, unsigned tag) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(tr.get(0));
  return sr_mix((unsigned)b ^ (unsigned)(b >> 32) ^ (tag * 0x9e3779b9u));
}

// b + c with dither r in [-1/2, 1/2): ulp(b) from b's exponent bits (zero for
// b = 0 and subnormals, where the addition is plain round-to-nearest).
__device__ __forceinline__ float add_sr(float b, float c, float r) {
  const int eb = (__float_as_int(b) & 0x7f800000) - (23 << 23);
  const float ulp = __int_as_float(eb > 0 ? eb : 0);
  return b + fmaf(r, ulp, c);
}

// Ten-bit dither number `slot` (0..2) from a 32-bit hash, in [-1/2, 1/2).
__device__ __forceinline__ float sr_draw(unsigned h, int slot) {
  return (float)((h >> (10 * slot)) & 1023u) * (1.0f / 1024.0f) - 0.5f;
}

// state + increment: stochastically rounded in float (h: the draw), exact
// IEEE addition otherwise.
template <typename T>
__device__ __forceinline__ T state_add(T b, T c, float r) {
  if constexpr (std::is_same<T, float>::value)
    return add_sr(b, c, r);
  else
    return b + c;
}

// include/MomentumEquation.h:42-116 (OPT_CPU_CACHE branch)
template <typename T>
__device__ __forceinline__ T rhs_u(const T *u, const T *v, const T *w, long q, long sy, long sz, const Coeffs<T> &c) {
  const T u13 = ld(u, q - 1), u11 = ld(u, q - sy), u5 = ld(u, q - sz), u14 = ld(u, q), u23 = ld(u, q + sz),
          u17 = ld(u, q + sy), u15 = ld(u, q + 1);
  const T v13 = ld(v, q - 1), v16 = ld(v, q - 1 + sy), v14 = ld(v, q), v17 = ld(v, q + sy);
  const T w13 = ld(w, q - 1), w22 = ld(w, q - 1 + sz), w14 = ld(w, q), w23 = ld(w, q + sz);
  const T conv = -u14 * (u15 - u13) * c.o2h[0] - (v17 + v14 + v16 + v13) * (u17 - u11) * c.o8h[1] -
                 (w23 + w14 + w22 + w13) * (u23 - u5) * c.o8h[2];
  const T diff = (u15 - T(2) * u14 + u13) * c.oh2Re[0] + (u17 - T(2) * u14 + u11) * c.oh2Re[1] +
                 (u23 - T(2) * u14 + u5) * c.oh2Re[2];
  return conv + diff;
}

// include/MomentumEquation.h:119-185
template <typename T>
__device__ __forceinline__ T rhs_v(const T *u, const T *v, const T *w, long q, long sy, long sz, const Coeffs<T> &c) {
  const T u11 = ld(u, q - sy), u14 = ld(u, q), u12 = ld(u, q + 1 - sy), u15 = ld(u, q + 1);
  const T v13 = ld(v, q - 1), v11 = ld(v, q - sy), v5 = ld(v, q - sz), v14 = ld(v, q), v23 = ld(v, q + sz),
          v17 = ld(v, q + sy), v15 = ld(v, q + 1);
  const T w11 = ld(w, q - sy), w20 = ld(w, q - sy + sz), w14 = ld(w, q), w23 = ld(w, q + sz);
  const T conv = -(u15 + u14 + u12 + u11) * (v15 - v13) * c.o8h[0] - v14 * (v17 - v11) * c.o2h[1] -
                 (w23 + w14 + w20 + w11) * (v23 - v5) * c.o8h[2];
  const T diff = (v15 - T(2) * v14 + v13) * c.oh2Re[0] + (v17 - T(2) * v14 + v11) * c.oh2Re[1] +
                 (v23 - T(2) * v14 + v5) * c.oh2Re[2];
  return conv + diff;
}

// include/MomentumEquation.h:188-255
template <typename T>
__device__ __forceinline__ T rhs_w(const T *u, const T *v, const T *w, long q, long sy, long sz, const Coeffs<T> &c) {
  const T u5 = ld(u, q - sz), u14 = ld(u, q), u6 = ld(u, q + 1 - sz), u15 = ld(u, q + 1);
  const T v5 = ld(v, q - sz), v14 = ld(v, q), v8 = ld(v, q + sy - sz), v17 = ld(v, q + sy);
  const T w13 = ld(w, q - 1), w11 = ld(w, q - sy), w5 = ld(w, q - sz), w14 = ld(w, q), w23 = ld(w, q + sz),
          w17 = ld(w, q + sy), w15 = ld(w, q + 1);
  const T conv = -(u15 + u14 + u6 + u5) * (w15 - w13) * c.o8h[0] - (v17 + v14 + v8 + v5) * (w17 - w11) * c.o8h[1] -
                 w14 * (w23 - w5) * c.o2h[2];
  const T diff = (w15 - T(2) * w14 + w13) * c.oh2Re[0] + (w17 - T(2) * w14 + w11) * c.oh2Re[1] +
                 (w23 - T(2) * w14 + w5) * c.oh2Re[2];
  return conv + diff;
}

// Momentum forcing of the SINCOS family at component c's staggered point,
// from per-axis sin/cos tables: f = u_t + (u.grad)u - lap(u)/Re
// (+ grad p), the residual generators/manufsol_velocity.py:32-50 derives.
template <typename T>
struct ForcingEval {
  const T *tab;
  int maxE;
  T st, ct, invRe;
  int with_p;
  int tg;   // Taylor-Green body force alpha (sin x cos y cos z, -cos x sin y cos z, 0) instead
  T alpha;
  __device__ __forceinline__ T S(int ax, int face, int i) const { return tab[((ax * 2 + face) * 2 + 0) * maxE + i]; }
  __device__ __forceinline__ T C(int ax, int face, int i) const { return tab[((ax * 2 + face) * 2 + 1) * maxE + i]; }
  // sin/cos at the node ([0]) and the face ([1]) coordinate of one index per axis.
  struct Axis {
    T s[2], c[2];
  };
  __device__ __forceinline__ Axis axis(int ax, int i) const {
    return Axis{{S(ax, 0, i), S(ax, 1, i)}, {C(ax, 0, i), C(ax, 1, i)}};
  }
  // Component c at the staggered point with per-axis factors X, Y, Z (the
  // x and y ones are constant through a thread's march in z).
  __device__ __forceinline__ T eval(int c, const Axis &X, const Axis &Y, const Axis &Z) const {
    const T sx = X.s[c == 0], cx = X.c[c == 0];
    const T sy = Y.s[c == 1], cy = Y.c[c == 1];
    const T sz = Z.s[c == 2], cz = Z.c[c == 2];
    T f;
    if (tg) return c == 0 ? alpha * (sx * cy * cz) : (c == 1 ? -alpha * (cx * sy * cz) : T(0));
    if (c == 0) {
      f = sx * cy * sz * ct + st * st * sx * cx * (cy * cy * sz * sz - sy * sy * sz * sz + T(2) * cy * cy * cz * cz) +
          T(3) * sx * cy * sz * st * invRe;
      if (with_p) f += -sx * cy * sz * st;
    } else if (c == 1) {
      f = cx * sy * sz * ct + st * st * sy * cy * (cx * cx * sz * sz - sx * sx * sz * sz + T(2) * cx * cx * cz * cz) +
          T(3) * cx * sy * sz * st * invRe;
      if (with_p) f += -cx * sy * sz * st;
    } else {
      f = T(2) * cx * cy * cz * ct -
          T(2) * st * st * sz * cz * (sx * sx * cy * cy + cx * cx * sy * sy + T(2) * cx * cx * cy * cy) +
          T(6) * cx * cy * cz * st * invRe;
      if (with_p) f += cx * cy * cz * st;
    }
    return f;
  }
};

template <typename T>
struct StageCoef {
  T k1, k2, k3, k4;
};

// ---- 2.5D-tiled stage kernel ----
//
// A CTA owns a TX x TY tile of (i, j) and marches through kc planes of k. The
// input velocity set and p live in a ring of four shared-memory planes per
// field (k-1, k, k+1 and the plane being prefetched), each with a one-point
// halo in x and y; plane k+2 is loaded by TMA while plane k is computed.
// Every stencil neighbour of include/MomentumEquation.h then comes from
// shared memory and each point costs about five global loads. Tile rows hold
// kTX + 2 used elements at a pitch of kTX + 4: a plane tile is one TMA box of
// kHX x kHY elements. A TMA destination in shared memory starts 128-byte
// aligned, so the ring slots are kSlot elements apart (the kPL-element tile
// and padding; 896 bytes in float, 1792 in double).
constexpr int kTX = 32, kTY = 4, kHX = kTX + 4, kHY = kTY + 2, kPL = kHX * kHY, kSlot = 224;
static_assert(kSlot >= kPL && (kSlot * 4) % 128 == 0, "128-byte aligned ring slots");

template <typename T>
struct Ring {
  T f[4][4][kSlot];  // field (u, v, w, p), slot (k & 3), tile
};

// Neighbour accessor on the ring: field f at (i + di, j + dj, k + dk).
template <typename T>
struct Tap {
  // pl[dk + 1]: this thread's point in the slot of plane k + dk (field 0);
  // field f is 4 slots further per field, so every read is a base pointer
  // plus a compile-time offset.
  const T *pl[3];
  __device__ __forceinline__ T operator()(int f, int di, int dj, int dk) const {
    return pl[dk + 1][f * 4 * kSlot + dj * kHX + di];
  }
};

// Every ring value the three momentum components and the pressure gradient
// read at one point (31 distinct taps), named by the reference's stencil
// numbering (include/MomentumEquation.h: 14 the point, 13/15 x-1/x+1,
// 11/17 y-1/y+1, 5/23 z-1/z+1, and the mixed corners). They are read once,
// before any store: the stores go to global memory through generic pointers,
// which the compiler cannot separate from the ring, so reads interleaved
// with them would be repeated per component.
template <typename T>
struct Taps {
  T u5, u6, u11, u12, u13, u14, u15, u17, u23;
  T v5, v8, v11, v13, v14, v15, v16, v17, v23;
  T w5, w11, w13, w14, w15, w17, w20, w22, w23;
  T p5, p11, p13, p14;
  __device__ __forceinline__ void load(const Tap<T> &A, bool with_p) {
    u13 = A(0, -1, 0, 0), u11 = A(0, 0, -1, 0), u5 = A(0, 0, 0, -1), u14 = A(0, 0, 0, 0), u23 = A(0, 0, 0, 1);
    u17 = A(0, 0, 1, 0), u15 = A(0, 1, 0, 0), u12 = A(0, 1, -1, 0), u6 = A(0, 1, 0, -1);
    v13 = A(1, -1, 0, 0), v16 = A(1, -1, 1, 0), v14 = A(1, 0, 0, 0), v17 = A(1, 0, 1, 0), v11 = A(1, 0, -1, 0);
    v5 = A(1, 0, 0, -1), v23 = A(1, 0, 0, 1), v15 = A(1, 1, 0, 0), v8 = A(1, 0, 1, -1);
    w13 = A(2, -1, 0, 0), w22 = A(2, -1, 0, 1), w14 = A(2, 0, 0, 0), w23 = A(2, 0, 0, 1), w11 = A(2, 0, -1, 0);
    w20 = A(2, 0, -1, 1), w5 = A(2, 0, 0, -1), w17 = A(2, 0, 1, 0), w15 = A(2, 1, 0, 0);
    if (with_p) p14 = A(3, 0, 0, 0), p13 = A(3, -1, 0, 0), p11 = A(3, 0, -1, 0), p5 = A(3, 0, 0, -1);
  }
  // Only the taps component c's right-hand side and pressure gradient read
  // (15 of the 31, plus two of p).
  __device__ __forceinline__ void load_c(const Tap<T> &A, int c, bool with_p) {
    if (c == 0) {
      u13 = A(0, -1, 0, 0), u11 = A(0, 0, -1, 0), u5 = A(0, 0, 0, -1), u14 = A(0, 0, 0, 0), u23 = A(0, 0, 0, 1);
      u17 = A(0, 0, 1, 0), u15 = A(0, 1, 0, 0);
      v13 = A(1, -1, 0, 0), v16 = A(1, -1, 1, 0), v14 = A(1, 0, 0, 0), v17 = A(1, 0, 1, 0);
      w13 = A(2, -1, 0, 0), w22 = A(2, -1, 0, 1), w14 = A(2, 0, 0, 0), w23 = A(2, 0, 0, 1);
      if (with_p) p14 = A(3, 0, 0, 0), p13 = A(3, -1, 0, 0);
    } else if (c == 1) {
      u14 = A(0, 0, 0, 0), u15 = A(0, 1, 0, 0), u12 = A(0, 1, -1, 0), u11 = A(0, 0, -1, 0);
      v13 = A(1, -1, 0, 0), v14 = A(1, 0, 0, 0), v17 = A(1, 0, 1, 0), v11 = A(1, 0, -1, 0);
      v5 = A(1, 0, 0, -1), v23 = A(1, 0, 0, 1), v15 = A(1, 1, 0, 0);
      w14 = A(2, 0, 0, 0), w23 = A(2, 0, 0, 1), w11 = A(2, 0, -1, 0), w20 = A(2, 0, -1, 1);
      if (with_p) p14 = A(3, 0, 0, 0), p11 = A(3, 0, -1, 0);
    } else {
      u5 = A(0, 0, 0, -1), u14 = A(0, 0, 0, 0), u15 = A(0, 1, 0, 0), u6 = A(0, 1, 0, -1);
      v5 = A(1, 0, 0, -1), v14 = A(1, 0, 0, 0), v17 = A(1, 0, 1, 0), v8 = A(1, 0, 1, -1);
      w13 = A(2, -1, 0, 0), w14 = A(2, 0, 0, 0), w23 = A(2, 0, 0, 1), w11 = A(2, 0, -1, 0);
      w5 = A(2, 0, 0, -1), w17 = A(2, 0, 1, 0), w15 = A(2, 1, 0, 0);
      if (with_p) p14 = A(3, 0, 0, 0), p5 = A(3, 0, 0, -1);
    }
  }
  __device__ __forceinline__ T self(int c) const { return c == 0 ? u14 : (c == 1 ? v14 : w14); }
  // p at the point minus p one step back along axis c
  __device__ __forceinline__ T dp(int c) const { return p14 - (c == 0 ? p13 : (c == 1 ? p11 : p5)); }
};

// include/MomentumEquation.h:42-255 (OPT_CPU_CACHE branch), term for term.
template <typename T>
__device__ __forceinline__ T rhs_taps(int c, const Taps<T> &a, const Coeffs<T> &co) {
  if (c == 0) {
    const T conv = -a.u14 * (a.u15 - a.u13) * co.o2h[0] - (a.v17 + a.v14 + a.v16 + a.v13) * (a.u17 - a.u11) * co.o8h[1] -
                   (a.w23 + a.w14 + a.w22 + a.w13) * (a.u23 - a.u5) * co.o8h[2];
    const T diff = (a.u15 - T(2) * a.u14 + a.u13) * co.oh2Re[0] + (a.u17 - T(2) * a.u14 + a.u11) * co.oh2Re[1] +
                   (a.u23 - T(2) * a.u14 + a.u5) * co.oh2Re[2];
    return conv + diff;
  }
  if (c == 1) {
    const T conv = -(a.u15 + a.u14 + a.u12 + a.u11) * (a.v15 - a.v13) * co.o8h[0] - a.v14 * (a.v17 - a.v11) * co.o2h[1] -
                   (a.w23 + a.w14 + a.w20 + a.w11) * (a.v23 - a.v5) * co.o8h[2];
    const T diff = (a.v15 - T(2) * a.v14 + a.v13) * co.oh2Re[0] + (a.v17 - T(2) * a.v14 + a.v11) * co.oh2Re[1] +
                   (a.v23 - T(2) * a.v14 + a.v5) * co.oh2Re[2];
    return conv + diff;
  }
  const T conv = -(a.u15 + a.u14 + a.u6 + a.u5) * (a.w15 - a.w13) * co.o8h[0] -
                 (a.v17 + a.v14 + a.v8 + a.v5) * (a.w17 - a.w11) * co.o8h[1] - a.w14 * (a.w23 - a.w5) * co.o2h[2];
  const T diff = (a.w15 - T(2) * a.w14 + a.w13) * co.oh2Re[0] + (a.w17 - T(2) * a.w14 + a.w11) * co.oh2Re[1] +
                 (a.w23 - T(2) * a.w14 + a.w5) * co.oh2Re[2];
  return conv + diff;
}

// Float: 48 warps per SM at 40 registers, with a few dozen bytes of spills;
// the march is latency bound (barriers, plane loads). On GB300 at 512^3, with
// the ring then filled by per-thread 16-byte cp.async copies, the plain float
// stage time per step measured 5.30 / 5.48 / 4.80 / 4.61 / 4.48 / 4.75 ms for
// 2 / 3 / 4 / 5 / 6 / 8 CTAs of 32 x 8 threads per SM, and 4.44 ms for twelve
// CTAs of 32 x 4 (half the threads per barrier, 20 % more halo rows). FP64:
// 8 warps per SM.
// kComp (float only, projection stages): the input state is hi + residual
// and the output state is written as an error-free sum (comp_add) into its
// float field and the residual, in place (Residual).
// Resident CTAs per SM the register budget is sized for: float, the
// compensated float variant, double.
constexpr int kStageMinBlocksF32 = 12, kStageMinBlocksComp = 12, kStageMinBlocksF64 = 4;
template <typename T, int ST, bool kComp>
__global__ void __launch_bounds__(kTX *kTY, sizeof(T) == 4 ? (kComp ? kStageMinBlocksComp : kStageMinBlocksF32)
                                                           : kStageMinBlocksF64)
    stage_kernel_tiled(Geometry g, Coeffs<T> co, Fields<T> F, StageCoef<T> K, int forcing, ForcingEval<T> fe,
                       TimeRef tr, int sin_slot, int kc, Residual res, const __grid_constant__ StageMaps maps,
                       int *kerr) {
  // maps.m[0..2]: the input set's u, v, w (set 0 for Y2 and the velocity-only
  // Y2 and U*, set 1 for Y3, set 2 for U* and the velocity-only Y3), m[3]: p
  constexpr bool kUseP = ST == kStageY2 || ST == kStageY3 || ST == kStageUStar;
  __shared__ __align__(128) Ring<T> ring;
  if (forcing) {
    fe.st = T(tr.get(sin_slot));
    fe.ct = T(tr.get(sin_slot + 1));
  }
  const unsigned salt = std::is_same<T, float>::value ? sr_salt(tr, 1u + ST) : 0u;
  const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
  const int i0 = 1 + blockIdx.x * kTX, j0 = 1 + blockIdx.y * kTY;
  const int zmax = g.Es[2] - 1;  // interior k < zmax
  const int kbeg = 1 + blockIdx.z * kc, kend = min(kbeg + kc, zmax);
  constexpr int nf = kUseP ? 4 : 3;
  // The ring is filled by TMA: thread 0 loads plane kk's nf tiles (36 x 6
  // elements from (i0 - 1, j0 - 1), i0 - 1 = 32 * blockIdx.x, 16-byte
  // aligned as PX is a multiple of 8; zeros outside the box) into slot
  // kk & 3 on that slot's mbarrier, and every thread waits on the barrier
  // before reading the plane. Plane kk is the ((kk - kfirst) / 4)-th load of
  // its slot, which fixes the phase to wait for.
  __shared__ uint64_t bars[4];
  const int kfirst = kbeg - 1;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int b = 0; b < 4; ++b) mbar_init(&bars[b], 1);
    mbar_init_fence();
  }
  __syncthreads();
  auto load_plane = [&](int kk) {  // thread 0
    uint64_t *bar = &bars[kk & 3];
    if (kk >= 0 && kk < g.PZ) {
      mbar_expect_tx(bar, (unsigned)(nf * kPL * sizeof(T)));
#pragma unroll
      for (int f = 0; f < nf; ++f) tma_load_3d(&ring.f[f][kk & 3][0], &maps.m[f], i0 - 1, j0 - 1, kk, bar);
    } else {
      mbar_arrive(bar);
    }
  };
  // A wait that gives up records it in *kerr; later waits of the thread are
  // skipped, so a CTA always runs to its end.
  bool tma_ok = true;
  auto wait_plane = [&](int kk) {
    if (tma_ok && !mbar_wait(&bars[kk & 3], ((kk - kfirst) >> 2) & 1)) {
      tma_ok = false;
      if (kerr) atomicExch(kerr, 1);
    }
  };
  if (threadIdx.x == 0) {
    load_plane(kbeg - 1);
    load_plane(kbeg);
    load_plane(kbeg + 1);
  }
  const int i = i0 + tx, j = j0 + ty;
  const long sy = g.sy(), sz = g.sz();
  const T *const tap0 = &ring.f[0][0][(ty + 1) * kHX + tx + 1];
  typename ForcingEval<T>::Axis fx{}, fy{}, fz{};
  if (forcing) {
    fx = fe.axis(0, min(i, fe.maxE - 1));
    fy = fe.axis(1, min(j, fe.maxE - 1));
  }
  // Point values of the other sets the update reads at (i, j, k) (set 2 in
  // Y3 and the velocity-only stages, set 0 in U* and the velocity-only Y3),
  // prefetched into registers one plane ahead so their latency hides behind
  // the stencil work.
  constexpr bool kPre2 = ST == kStageY3 || ST == kVelY3 || ST == kVelUStar;
  constexpr bool kPre0 = ST == kStageUStar || ST == kVelY3;
  const bool in_box = i < g.PX && j < g.PY;
  T n2[3] = {T(0), T(0), T(0)}, n0[3] = {T(0), T(0), T(0)};
  // the input state's residual at the point, prefetched the same way
  __nv_bfloat16 nl[3] = {__float2bfloat16_rn(0.f), __float2bfloat16_rn(0.f), __float2bfloat16_rn(0.f)};
  auto prefetch = [&](int kk) {
    if (!in_box || kk >= kend) return;
    const long qq = g.idx(i, j, kk);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (kPre2) n2[c] = F.vel(2, c)[qq];
      if (kPre0) n0[c] = F.vel(0, c)[qq];
      if constexpr (kComp) nl[c] = res.c[c][qq];
    }
  };
  prefetch(kbeg);
  // Per-thread invariants of the march: which components have (i, j) inside
  // their interior, their last interior plane, and the (i, j) offset.
  bool own_ij[3];
  int klim[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    own_ij[c] = i < g.ext(c, 0) - 1 && j < g.ext(c, 1) - 1;
    klim[c] = g.ext(c, 2) - 1;
  }
  const long qij = (long)i + g.PX * (long)j;
  wait_plane(kbeg - 1);
  wait_plane(kbeg);
  for (int k = kbeg; k < kend; ++k) {
    // plane k + 2 into the slot of plane k - 2, which the barrier that ended
    // the previous iteration released
    if (threadIdx.x == 0 && k + 2 <= kend) {
      fence_async_shared();
      load_plane(k + 2);
    }
    if (forcing) fz = fe.axis(2, k);
    T c2[3], c0[3];
    __nv_bfloat16 cl[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      c2[c] = n2[c];
      c0[c] = n0[c];
      cl[c] = nl[c];
    }
    prefetch(k + 1);
    wait_plane(k + 1);
    Tap<T> A;
#pragma unroll
    for (int dk = -1; dk <= 1; ++dk) A.pl[dk + 1] = tap0 + ((k + dk) & 3) * kSlot;
    const long q = qij + (long)k * sz;
    const unsigned hq = std::is_same<T, float>::value ? sr_mix((unsigned)q ^ salt) : 0u;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (!own_ij[c] || k >= klim[c]) continue;
      // each component's taps are read right before its update: the global
      // stores of the previous component keep the compiler from hoisting
      // them, so at most one component's taps are live (no spills)
      Taps<T> tp;
      tp.load_c(A, c, kUseP);
      T r = rhs_taps(c, tp, co);
      if (forcing) r = r + fe.eval(c, fx, fy, fz);
      T gp = T(0);
      if (kUseP) gp = tp.dp(c) * co.oh[c];
      const T self = tp.self(c);  // the input set's own value at the point
      if constexpr (kComp) {
        // the same increments as below, added to hi + residual without loss
        const float lo = __bfloat162float(cl[c]);
        __nv_bfloat16 *lo_out = res.c[c] + q;
        if constexpr (ST == kStageY2) {
          F.vel(1, c)[q] = comp_add(self, lo, K.k1 * r - K.k3 * gp, lo_out);
          F.vel(2, c)[q] = r;
        } else if constexpr (ST == kStageY3) {
          const T r2s = K.k2 * r;
          F.vel(2, c)[q] = comp_add(self, lo, K.k1 * c2[c] + r2s - K.k3 * gp, lo_out);
          F.vel(0, c)[q] = r2s;
        } else {
          F.vel(0, c)[q] = comp_add(self, lo, -c0[c] + K.k2 * r - K.k3 * gp, lo_out);
        }
        continue;
      }
      // FP64 keeps the reference's expression order; the float path adds the
      // increment to the state with stochastic rounding
      constexpr bool kSR = std::is_same<T, float>::value;
      const float h = kSR ? sr_draw(hq, c) : 0.f;
      if (ST == kStageY2) {
        F.vel(1, c)[q] = kSR ? state_add(self, K.k1 * r - K.k3 * gp, h) : self + K.k1 * r - K.k3 * gp;
        F.vel(2, c)[q] = r;
      } else if (ST == kStageY3) {
        const T r1 = c2[c];
        const T r2s = K.k2 * r;
        F.vel(2, c)[q] = kSR ? state_add(self, K.k1 * r1 + r2s - K.k3 * gp, h) : self + K.k1 * r1 + r2s - K.k3 * gp;
        F.vel(0, c)[q] = r2s;
      } else if (ST == kStageUStar) {
        const T r2s = -c0[c];
        F.vel(0, c)[q] = kSR ? state_add(self, r2s + K.k2 * r - K.k3 * gp, h) : self + r2s + K.k2 * r - K.k3 * gp;
      } else if (ST == kVelY2) {
        F.vel(2, c)[q] = r;
        F.vel(1, c)[q] = kSR ? state_add(self, K.k1 * r, h) : self + K.k1 * r;
      } else if (ST == kVelY3) {
        const T r1 = c2[c];
        const T uu = c0[c];
        F.vel(2, c)[q] = kSR ? state_add(uu, K.k1 * (K.k2 * r1), h) : uu + K.k1 * (K.k2 * r1);
        F.vel(0, c)[q] = kSR ? state_add(uu, K.k1 * (K.k3 * r1 + K.k4 * r), -h) : uu + K.k1 * (K.k3 * r1 + K.k4 * r);
      } else {
        const T r1 = c2[c];
        F.vel(1, c)[q] = kSR ? state_add(r1, K.k1 * (K.k2 * r), h) : r1 + K.k1 * (K.k2 * r);
      }
    }
    __syncthreads();  // the next iteration refills the slot of plane k - 1
  }
  (void)sy;
  (void)sz;
}

// ---- compensated stage with the previous projection inside ----
//
// In the compensated state the projections that follow the Y2 and Y3 stages
// (src/Timestep.cpp:97-141) are applied by the next stage kernel to its own
// plane ring, as each plane arrives. The projected set is read by that next
// stage only, so the projected velocity never goes back to memory: per step
// this saves two projection passes (the velocity and residual read and
// written, twelve float sweeps each) for one more ring field (phi) and the
// pressure update, written here. Between the steps of one run the step's
// last projection is applied the same way by the next step's Y2 stage.
//
// Ring values: u' = fl(u + inc), inc = (phi_b - phi) * (oh * dt) with
// phi_b the neighbour one step back along the component's axis, on the
// points project_pair_kernel updates (interior of the component), the others
// as they are. The stencils read these float values as they read the
// projected float field. The state update needs the exact projected state at
// the thread's own point: projecting a plane, the thread splits its own
// point's u + inc into u' + e (TwoSum) and keeps lo' = lo + e beside u' (lo
// the stored residual), so the update adds its increment to u' + lo' with
// comp_add as the unfused stage does.
//
// The pressure p + phi is written stochastically rounded, as
// project_pair_kernel writes it, into p_out: other CTAs still read p_in as halo. The
// pressure gradient of the stage uses (p + phi) unrounded, as the difference of
// p plus the difference of phi. Pressure nodes outside the threads' range
// (x = 0, y = 0, z = 0 and the last x node of a periodic axis when it falls on
// the tile halo) are written by the CTAs at those edges.

// phi tile: one TMA box of kPhiX x kPhiRows from (i0 - 5, j0 - 2), 16-byte
// aligned in x: ring point (hx, hy) is phi element (hx + 4, hy + 1).
constexpr int kPhiRows = kTY + 3, kPhiX = kHX + 4, kPhiPL = kPhiX * kPhiRows, kPhiSlot = 288;
static_assert(kPhiSlot >= kPhiPL && (kPhiSlot * 4) % 128 == 0, "128-byte aligned phi slots");
struct RingProj {
  float f[4][4][kSlot];  // u, v, w, p: slot (k & 3), as Ring
  float phi[4][kPhiSlot];
};
// The ring points (hx, hy) outside the CTA's own kTX x kTY: rows hy = 0 and
// kTY + 1 (hx = 1 .. kTX), then columns hx = 0 and kTX + 1 (hy = 0 .. kTY + 1).
constexpr int kHaloPts = 2 * kTX + 2 * (kTY + 2);
// Resident CTAs per SM the register budget is sized for. The kernel is
// issue-bound (about 750 instructions per point): on GB300 at 512^3 its time
// was the same at 12, 10 and 8 CTAs per SM with the same spills, and 8 CTAs
// (64 registers) remove the spills (40 registers: ~100 bytes a thread, 22
// local loads per warp and point), which took the two stages from 2.67 to
// 2.48 ms each.
#ifndef MIFGPU_STAGE_PROJ_BLOCKS
#define MIFGPU_STAGE_PROJ_BLOCKS 8
#endif
constexpr int kStageProjMinBlocks = MIFGPU_STAGE_PROJ_BLOCKS;

template <int ST, bool kForce>
__global__ void __launch_bounds__(kTX *kTY, kStageProjMinBlocks)
    stage_proj_kernel(Geometry g, Coeffs<float> co, Fields<float> F, StageCoef<float> K, ForcingEval<float> fe,
                      TimeRef tr, int sin_slot, int kc, Residual res, StageProj pj,
                      const __grid_constant__ StageMaps maps, int *kerr) {
  static_assert(ST == kStageY2 || ST == kStageY3 || ST == kStageUStar, "the projection stages");
  // the other set read at the own point: set 2 (Y2's right-hand side) for Y3,
  // set 0 (Y3's scaled one) for U*; Y2 reads none
  constexpr bool kOth = ST != kStageY2;
  constexpr int oth_set = ST == kStageY3 ? 2 : 0;
  __shared__ __align__(128) RingProj ring;
  __shared__ uint64_t bars[4];
  if (kForce) {
    fe.st = float(tr.get(sin_slot));
    fe.ct = float(tr.get(sin_slot + 1));
  }
  // Parameters the plane loop uses, as locals (the lambdas below capture
  // locals only).
  const long plane = g.sz(), PX = g.PX;
  const int PZ = (int)g.PZ;
  const int lim0 = g.ext(0, 2) - 1, lim1 = g.ext(1, 2) - 1, lim2 = g.ext(2, 2) - 1;
  const float oh0 = co.oh[0], oh1 = co.oh[1], oh2 = co.oh[2];
  // the projection increment (phi_b - phi) * oh * dt, with oh * dt formed once
  const float cd0 = oh0 * pj.dt, cd1 = oh1 * pj.dt, cd2 = oh2 * pj.dt;
  float *const p_out = pj.p_out;
  const int tid = threadIdx.x, tx = tid % kTX, ty = tid / kTX;
  const int i0 = 1 + blockIdx.x * kTX, j0 = 1 + blockIdx.y * kTY;
  const int zmax = g.Es[2] - 1;  // interior k < zmax
  const int kbeg = 1 + blockIdx.z * kc, kend = min(kbeg + kc, zmax);
  // TMA ring fill (as stage_kernel_tiled): maps 0..3 the input set's u, v, w
  // and p_in (kHX x kHY boxes from (i0 - 1, j0 - 1)), map 4 phi (kPhiX x
  // kPhiRows from (i0 - 5, j0 - 2)); thread 0 loads, every thread waits on the
  // slot's mbarrier. The first load is phi alone, of plane kbeg - 2.
  const int kfirst = kbeg - 2;
  if (tid == 0) {
#pragma unroll
    for (int b = 0; b < 4; ++b) mbar_init(&bars[b], 1);
    mbar_init_fence();
  }
  __syncthreads();
  auto load_plane = [&](int kk, bool phi_only) {  // thread 0
    uint64_t *bar = &bars[kk & 3];
    if (kk >= 0 && kk < PZ) {
      mbar_expect_tx(bar, (unsigned)(sizeof(float) * (kPhiPL + (phi_only ? 0 : 4 * kPL))));
      if (!phi_only)
#pragma unroll
        for (int f = 0; f < 4; ++f) tma_load_3d(&ring.f[f][kk & 3][0], &maps.m[f], i0 - 1, j0 - 1, kk, bar);
      tma_load_3d(&ring.phi[kk & 3][0], &maps.m[4], i0 - 5, j0 - 2, kk, bar);
    } else {
      mbar_arrive(bar);
    }
  };
  bool tma_ok = true;
  auto wait_plane = [&](int kk) {
    if (tma_ok && !mbar_wait(&bars[kk & 3], ((kk - kfirst) >> 2) & 1)) {
      tma_ok = false;
      if (kerr) atomicExch(kerr, 1);
    }
  };
  const int i = i0 + tx, j = j0 + ty;
  typename ForcingEval<float>::Axis fx{}, fy{}, fz{};
  if (kForce) {
    fx = fe.axis(0, min(i, fe.maxE - 1));
    fy = fe.axis(1, min(j, fe.maxE - 1));
  }
  // The other set's value at the point (set 2 for Y3, set 0 for U*) and the
  // input state's stored residual, prefetched one plane ahead.
  const bool in_box = i < PX && j < g.PY;
  const long qij = (long)i + PX * (long)j;
  const float *const oth0 = F.vel(oth_set, 0) + qij, *const oth1 = F.vel(oth_set, 1) + qij,
                     *const oth2 = F.vel(oth_set, 2) + qij;
  const __nv_bfloat16 *const res0 = res.c[0] + qij, *const res1 = res.c[1] + qij, *const res2 = res.c[2] + qij;
  float n0 = 0.f, n1 = 0.f, n2 = 0.f;
  __nv_bfloat16 l0 = __float2bfloat16_rn(0.f), l1 = l0, l2 = l0;
  auto prefetch = [&](int kk) {
    if (!in_box || kk >= kend) return;
    const long po = (long)kk * plane;
    if (kOth) {
      n0 = oth0[po];
      n1 = oth1[po];
      n2 = oth2[po];
    }
    l0 = res0[po];
    l1 = res1[po];
    l2 = res2[po];
  };
  // Interior masks in x and y of the own point (bits 0-2: component) and of
  // this thread's halo point (bits 3-5; threads < kHaloPts), whose ring index
  // is h_r and phi index h_p.
  int h_r = 0, h_p = 0;
  unsigned msk = 0;
  {
    int hx = 0, hy = 0;
    if (tid < kTX) hx = tid + 1, hy = 0;
    else if (tid < 2 * kTX) hx = tid - kTX + 1, hy = kTY + 1;
    else if (tid < 2 * kTX + kTY + 2) hx = 0, hy = tid - 2 * kTX;
    else hx = kTX + 1, hy = tid - 2 * kTX - (kTY + 2);
    h_r = hy * kHX + hx;
    h_p = (hy + 1) * kPhiX + hx + 4;
    const int hi_ = i0 - 1 + hx, hj = j0 - 1 + hy;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (i < g.ext(c, 0) - 1 && j < g.ext(c, 1) - 1) msk |= 1u << c;
      if (tid < kHaloPts && hi_ >= 1 && hj >= 1 && hi_ < g.ext(c, 0) - 1 && hj < g.ext(c, 1) - 1) msk |= 8u << c;
    }
  }
  const int o_r = (ty + 1) * kHX + tx + 1, o_p = (ty + 2) * kPhiX + tx + 5;  // own ring / phi index
  float e0 = 0.f, e1 = 0.f, e2 = 0.f;  // the own point's exact residuals at the plane projected last
  // Projection of ring plane kk: u' = fl(u + inc) at the interior points;
  // with own_exact the own point's stored residual lo becomes lo + e (e0..e2).
  auto two_sum_err = [](float a, float b, float s) {
    const float bb = __fsub_rn(s, a);
    return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  };
  auto project_plane = [&](int kk, bool own_exact) {
    float *const rb = ring.f[0][kk & 3];
    const float *const ph = ring.phi[kk & 3], *const phb = ring.phi[(kk - 1) & 3];
    const unsigned kin = (kk >= 1) ? ((kk < lim0 ? 9u : 0u) | (kk < lim1 ? 18u : 0u) | (kk < lim2 ? 36u : 0u)) : 0u;
    const unsigned m = msk & kin;
    {
      const float f0 = ph[o_p];
      float lo0 = __bfloat162float(l0), lo1 = __bfloat162float(l1), lo2 = __bfloat162float(l2);
      if (m & 1u) {
        const float inc = (ph[o_p - 1] - f0) * cd0, hi = rb[o_r], s = __fadd_rn(hi, inc);
        rb[o_r] = s;
        lo0 = __fadd_rn(lo0, two_sum_err(hi, inc, s));
      }
      if (m & 2u) {
        const float inc = (ph[o_p - kPhiX] - f0) * cd1, hi = rb[4 * kSlot + o_r], s = __fadd_rn(hi, inc);
        rb[4 * kSlot + o_r] = s;
        lo1 = __fadd_rn(lo1, two_sum_err(hi, inc, s));
      }
      if (m & 4u) {
        const float inc = (phb[o_p] - f0) * cd2, hi = rb[8 * kSlot + o_r], s = __fadd_rn(hi, inc);
        rb[8 * kSlot + o_r] = s;
        lo2 = __fadd_rn(lo2, two_sum_err(hi, inc, s));
      }
      if (own_exact) e0 = lo0, e1 = lo1, e2 = lo2;
    }
    if (m & 0x38u) {
      const float f0 = ph[h_p];
      if (m & 8u) rb[h_r] = __fadd_rn(rb[h_r], (ph[h_p - 1] - f0) * cd0);
      if (m & 16u) rb[4 * kSlot + h_r] = __fadd_rn(rb[4 * kSlot + h_r], (ph[h_p - kPhiX] - f0) * cd1);
      if (m & 32u) rb[8 * kSlot + h_r] = __fadd_rn(rb[8 * kSlot + h_r], (phb[h_p] - f0) * cd2);
    }
  };
  // p + phi, stochastically rounded (one hash round of the point and the
  // projection's salt gives the dither)
  const unsigned psalt = sr_salt(tr, pj.tag);
  auto p_new = [&](int r, int rp, int kk, long q) {
    return add_sr(ring.f[3][kk & 3][r], ring.phi[kk & 3][rp], sr_draw(sr_mix((unsigned)q ^ psalt), 0));
  };
  // Pressure nodes outside the threads' range, at the CTAs on those edges.
  const int E0 = g.E[0], E1 = g.E[1], E2 = g.E[2];
  // the last node E0 - 1 is the right halo only of the last tile (else a
  // later tile owns it)
  const bool edge_x0 = blockIdx.x == 0, edge_y0 = blockIdx.y == 0,
             edge_xr = i0 + kTX == E0 - 1 && blockIdx.x + 1 == gridDim.x;
  auto write_p_edges = [&](int kk) {
    auto one = [&](int hx, int hy) {
      const int pi = i0 - 1 + hx, pjj = j0 - 1 + hy;
      if (pi >= E0 || pjj >= E1 || kk >= E2) return;
      const long q = pi + PX * (pjj + g.PY * (long)kk);
      p_out[q] = p_new(hy * kHX + hx, (hy + 1) * kPhiX + hx + 4, kk, q);
    };
    if (edge_x0 && tx == 0) one(0, ty + 1);
    if (edge_xr && tx == kTX - 1) one(kTX + 1, ty + 1);
    if (edge_y0 && ty == 0) {
      one(tx + 1, 0);
      if (edge_x0 && tx == 0) one(0, 0);
      if (edge_xr && tx == kTX - 1) one(kTX + 1, 0);
    }
  };
  const bool own_p = i < E0 && j < E1;
  const bool edges = edge_x0 | edge_y0 | edge_xr;
  // Prologue: phi of plane kbeg - 2 (w's projection of plane kbeg - 1), the
  // planes kbeg - 1 .. kbeg + 1; planes kbeg - 1 and kbeg projected.
  if (tid == 0) {
    load_plane(kbeg - 2, true);
    load_plane(kbeg - 1, false);
    load_plane(kbeg, false);
    load_plane(kbeg + 1, false);
  }
  wait_plane(kbeg - 2);
  wait_plane(kbeg - 1);
  wait_plane(kbeg);
  project_plane(kbeg - 1, false);
  prefetch(kbeg);
  project_plane(kbeg, true);
  if (kbeg == 1) {  // the pressure of plane 0, which no thread's march reaches
    if (own_p) p_out[qij] = p_new(o_r, o_p, 0, qij);
    if (edges) write_p_edges(0);
  }
  __syncthreads();  // the first iteration refills the slot of plane kbeg - 2
  const float *const tap0 = &ring.f[0][0][o_r];
  for (int k = kbeg; k < kend; ++k) {
    if (tid == 0 && k + 2 <= kend) {
      fence_async_shared();
      load_plane(k + 2, false);
    }
    if (kForce) fz = fe.axis(2, k);
    const float c0 = n0, c1 = n1, c2 = n2, lo0 = e0, lo1 = e1, lo2 = e2;
    prefetch(k + 1);
    wait_plane(k + 1);
    project_plane(k + 1, true);
    __syncthreads();
    Tap<float> A;
#pragma unroll
    for (int dk = -1; dk <= 1; ++dk) A.pl[dk + 1] = tap0 + ((k + dk) & 3) * kSlot;
    const float *const ph = ring.phi[k & 3], *const phb = ring.phi[(k - 1) & 3];
    const float f14 = ph[o_p];
    const long q = qij + (long)k * plane;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (!((msk >> c) & 1u) || k >= (c == 0 ? lim0 : (c == 1 ? lim1 : lim2))) continue;
      Taps<float> tp;
      tp.load_c(A, c, true);
      float r = rhs_taps(c, tp, co);
      if (kForce) r = r + fe.eval(c, fx, fy, fz);
      const float fb = c == 0 ? ph[o_p - 1] : (c == 1 ? ph[o_p - kPhiX] : phb[o_p]);
      const float gp = (tp.dp(c) + (f14 - fb)) * (c == 0 ? oh0 : (c == 1 ? oh1 : oh2));
      const float self = tp.self(c);
      const float cur = c == 0 ? c0 : (c == 1 ? c1 : c2), lo = c == 0 ? lo0 : (c == 1 ? lo1 : lo2);
      __nv_bfloat16 *lo_out = res.c[c] + q;
      if constexpr (ST == kStageY2) {
        F.vel(1, c)[q] = comp_add(self, lo, K.k1 * r - K.k3 * gp, lo_out);
        F.vel(2, c)[q] = r;
        (void)cur;
      } else if constexpr (ST == kStageY3) {
        const float r2s = K.k2 * r;
        F.vel(2, c)[q] = comp_add(self, lo, K.k1 * cur + r2s - K.k3 * gp, lo_out);
        F.vel(0, c)[q] = r2s;
      } else {
        F.vel(0, c)[q] = comp_add(self, lo, -cur + K.k2 * r - K.k3 * gp, lo_out);
      }
    }
    if (own_p) p_out[q] = p_new(o_r, o_p, k, q);
    if (edges) write_p_edges(k);
    __syncthreads();  // the next iteration refills the slot of plane k - 1
  }
}

// ---- compensated projecting stage, two points per thread ----
//
// stage_proj_kernel's stage with each thread owning the two x-adjacent points
// (i, i + 1), i = i0 + 2 tx odd (i0 = 1 + 64 blockIdx.x): a CTA tile is
// 64 x 4 points, and a row of 512 interior points is eight tiles. The two
// points' arithmetic runs as packed two-lane float operations (add, mul and
// fma on float2, one instruction for both points, each lane rounded as the
// scalar operation), and the per-thread work (plane waits, masks, addresses,
// the dither hash) is shared by the pair. The stage kernels are issue-bound,
// so their instruction count sets their time.
// Ring rows are 72 elements from x = i0 - 5 (a multiple of 64 minus 4: the
// TMA box starts 16-byte aligned), so the own points sit at hx = 5 + 2 tx and
// 6 + 2 tx: a pair of taps one point back or ahead in x starts at an even
// index and is one 8-byte shared-memory load. The pair's global elements
// start at an odd index, so they move as single floats.
constexpr int kQX = 2 * kTX, kQHX = kQX + 8, kQPL = kQHX * kHY, kQSlot = 448;
constexpr int kQPhiPL = kQHX * kPhiRows, kQPhiSlot = 512;
static_assert(kQSlot >= kQPL && kQPhiSlot >= kQPhiPL && (kQSlot * 4) % 128 == 0 && (kQPhiSlot * 4) % 128 == 0,
              "128-byte aligned ring slots");
struct RingPair {
  float f[4][4][kQSlot];  // u, v, w, p: slot (k & 3); ring point (hx, hy) at hy * kQHX + hx
  float phi[4][kQPhiSlot];  // phi box from (i0 - 5, j0 - 2): ring point (hx, hy) at (hy + 1) * kQHX + hx
};
// Halo work per plane: rows hy = 0 and kTY + 1 as 32 pairs each (threads
// 0 .. 63), columns hx = 4 and kQX + 5 for hy = 0 .. kTY + 1 as single
// points (threads 64 .. 75).
constexpr int kQHaloCols = 2 * (kTY + 2);
// Resident CTAs per SM: six (36.9 KB of ring each; 80 registers a thread).
// At 512^3 the stage class measured the same within 1 % at five CTAs.
#ifndef MIFGPU_STAGE_PAIR_BLOCKS
#define MIFGPU_STAGE_PAIR_BLOCKS 6
#endif
constexpr int kStagePairMinBlocks = MIFGPU_STAGE_PAIR_BLOCKS;

__device__ __forceinline__ float2 splat2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b, rounded once: b * (-1) + a is exact before the rounding.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
// TwoSum's error of s = fl(a + b), lane by lane.
__device__ __forceinline__ float2 two_sum_err2(float2 a, float2 b, float2 s) {
  const float2 bb = sub2(s, a);
  return add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}
// comp_add for a pair: hi + (lo + inc) as an error-free sum; the error in err.
__device__ __forceinline__ float2 comp_add2(float2 hi, float2 lo, float2 inc, float2 &err) {
  const float2 t = add2(lo, inc);
  const float2 s = add2(hi, t);
  err = two_sum_err2(hi, t, s);
  return s;
}
// add_sr for a pair: b + c with dithers r (each in [-1/2, 1/2)) of ulp(b).
__device__ __forceinline__ float2 add_sr2(float2 b, float2 c, float2 r) {
  const int ea = (__float_as_int(b.x) & 0x7f800000) - (23 << 23), eb = (__float_as_int(b.y) & 0x7f800000) - (23 << 23);
  const float2 ulp = make_float2(__int_as_float(ea > 0 ? ea : 0), __int_as_float(eb > 0 ? eb : 0));
  return add2(b, fma2(r, ulp, c));
}
// Two consecutive ring elements from an even index (one 8-byte load) or from any.
__device__ __forceinline__ float2 lda2(const float *s, int o) { return *reinterpret_cast<const float2 *>(s + o); }
__device__ __forceinline__ float2 ldp2(const float *s, int o) { return make_float2(s[o], s[o + 1]); }

// The momentum right-hand side of component c at the pair, from the ring
// planes k - 1, k, k + 1 (m, z, p) of u, v, w at the pair's ring index o
// (odd), include/MomentumEquation.h:42-255 term for term; also returns the
// pair's own value (self) and p minus p one point back along c (dp).
template <int C>
__device__ __forceinline__ float2 rhs_pair(const float *const *U, const float *const *V, const float *const *W,
                                           const float *const *P, int o, const Coeffs<float> &co, float2 &self,
                                           float2 &dp) {
  constexpr int R = kQHX;
  float2 conv, diff;
  if constexpr (C == 0) {
    const float2 u13 = lda2(U[1], o - 1), u15 = lda2(U[1], o + 1), u14 = make_float2(u13.y, u15.x);
    const float2 u11 = ldp2(U[1], o - R), u17 = ldp2(U[1], o + R), u5 = ldp2(U[0], o), u23 = ldp2(U[2], o);
    const float2 v13 = lda2(V[1], o - 1), v14 = make_float2(v13.y, V[1][o + 1]);
    const float2 v16 = lda2(V[1], o - 1 + R), v17 = make_float2(v16.y, V[1][o + 1 + R]);
    const float2 w13 = lda2(W[1], o - 1), w14 = make_float2(w13.y, W[1][o + 1]);
    const float2 w22 = lda2(W[2], o - 1), w23 = make_float2(w22.y, W[2][o + 1]);
    const float2 p13 = lda2(P[1], o - 1), p14 = make_float2(p13.y, P[1][o + 1]);
    const float2 a = mul2(mul2(u14, sub2(u15, u13)), splat2(co.o2h[0]));
    const float2 b = mul2(mul2(add2(add2(add2(v17, v14), v16), v13), sub2(u17, u11)), splat2(co.o8h[1]));
    const float2 c = mul2(mul2(add2(add2(add2(w23, w14), w22), w13), sub2(u23, u5)), splat2(co.o8h[2]));
    conv = add2(add2(a, b), c);
    const float2 m2 = splat2(-2.f);
    diff = mul2(add2(fma2(u14, m2, u15), u13), splat2(co.oh2Re[0]));
    diff = fma2(add2(fma2(u14, m2, u17), u11), splat2(co.oh2Re[1]), diff);
    diff = fma2(add2(fma2(u14, m2, u23), u5), splat2(co.oh2Re[2]), diff);
    self = u14;
    dp = sub2(p14, p13);
  } else if constexpr (C == 1) {
    const float2 u15 = lda2(U[1], o + 1), u14 = make_float2(U[1][o], u15.x);
    const float2 u12 = lda2(U[1], o + 1 - R), u11 = make_float2(U[1][o - R], u12.x);
    const float2 v13 = lda2(V[1], o - 1), v15 = lda2(V[1], o + 1), v14 = make_float2(v13.y, v15.x);
    const float2 v11 = ldp2(V[1], o - R), v17 = ldp2(V[1], o + R), v5 = ldp2(V[0], o), v23 = ldp2(V[2], o);
    const float2 w14 = ldp2(W[1], o), w23 = ldp2(W[2], o), w11 = ldp2(W[1], o - R), w20 = ldp2(W[2], o - R);
    const float2 p14 = ldp2(P[1], o), p11 = ldp2(P[1], o - R);
    const float2 a = mul2(mul2(add2(add2(add2(u15, u14), u12), u11), sub2(v15, v13)), splat2(co.o8h[0]));
    const float2 b = mul2(mul2(v14, sub2(v17, v11)), splat2(co.o2h[1]));
    const float2 c = mul2(mul2(add2(add2(add2(w23, w14), w20), w11), sub2(v23, v5)), splat2(co.o8h[2]));
    conv = add2(add2(a, b), c);
    const float2 m2 = splat2(-2.f);
    diff = mul2(add2(fma2(v14, m2, v15), v13), splat2(co.oh2Re[0]));
    diff = fma2(add2(fma2(v14, m2, v17), v11), splat2(co.oh2Re[1]), diff);
    diff = fma2(add2(fma2(v14, m2, v23), v5), splat2(co.oh2Re[2]), diff);
    self = v14;
    dp = sub2(p14, p11);
  } else {
    const float2 u15 = lda2(U[1], o + 1), u14 = make_float2(U[1][o], u15.x);
    const float2 u6 = lda2(U[0], o + 1), u5 = make_float2(U[0][o], u6.x);
    const float2 v5 = ldp2(V[0], o), v14 = ldp2(V[1], o), v17 = ldp2(V[1], o + R), v8 = ldp2(V[0], o + R);
    const float2 w13 = lda2(W[1], o - 1), w15 = lda2(W[1], o + 1), w14 = make_float2(w13.y, w15.x);
    const float2 w11 = ldp2(W[1], o - R), w17 = ldp2(W[1], o + R), w5 = ldp2(W[0], o), w23 = ldp2(W[2], o);
    const float2 p14 = ldp2(P[1], o), p5 = ldp2(P[0], o);
    const float2 a = mul2(mul2(add2(add2(add2(u15, u14), u6), u5), sub2(w15, w13)), splat2(co.o8h[0]));
    const float2 b = mul2(mul2(add2(add2(add2(v17, v14), v8), v5), sub2(w17, w11)), splat2(co.o8h[1]));
    const float2 c = mul2(mul2(w14, sub2(w23, w5)), splat2(co.o2h[2]));
    conv = add2(add2(a, b), c);
    const float2 m2 = splat2(-2.f);
    diff = mul2(add2(fma2(w14, m2, w15), w13), splat2(co.oh2Re[0]));
    diff = fma2(add2(fma2(w14, m2, w17), w11), splat2(co.oh2Re[1]), diff);
    diff = fma2(add2(fma2(w14, m2, w23), w5), splat2(co.oh2Re[2]), diff);
    self = w14;
    dp = sub2(p14, p5);
  }
  return sub2(diff, conv);
}

template <int ST>
__global__ void __launch_bounds__(kTX *kTY, kStagePairMinBlocks)
    stage_pair_kernel(Geometry g, Coeffs<float> co, Fields<float> F, StageCoef<float> K, TimeRef tr, int kc,
                      Residual res, StageProj pj, const __grid_constant__ StageMaps maps, int *kerr) {
  static_assert(ST == kStageY2 || ST == kStageY3 || ST == kStageUStar, "the projection stages");
  constexpr bool kOth = ST != kStageY2;
  constexpr int oth_set = ST == kStageY3 ? 2 : 0;
  __shared__ __align__(128) RingPair ring;
  __shared__ uint64_t bars[4];
  const long plane = g.sz(), PX = g.PX;
  const int PZ = (int)g.PZ;
  const int lim0 = g.ext(0, 2) - 1, lim1 = g.ext(1, 2) - 1, lim2 = g.ext(2, 2) - 1;
  const float oh0 = co.oh[0], oh1 = co.oh[1], oh2 = co.oh[2];
  const float2 cd0 = splat2(oh0 * pj.dt), cd1 = splat2(oh1 * pj.dt), cd2 = splat2(oh2 * pj.dt);
  float *const p_out = pj.p_out;
  const int tid = threadIdx.x, tx = tid % kTX, ty = tid / kTX;
  const int i0 = 1 + blockIdx.x * kQX, j0 = 1 + blockIdx.y * kTY;
  const int zmax = g.Es[2] - 1;  // interior k < zmax
  const int kbeg = 1 + blockIdx.z * kc, kend = min(kbeg + kc, zmax);
  // TMA ring fill as stage_proj_kernel's, with kQHX-wide boxes from
  // x = i0 - 5: maps 0..3 the input set's u, v, w and p_in (rows from
  // j0 - 1), map 4 phi (kPhiRows rows from j0 - 2).
  const int kfirst = kbeg - 2;
  if (tid == 0) {
#pragma unroll
    for (int b = 0; b < 4; ++b) mbar_init(&bars[b], 1);
    mbar_init_fence();
  }
  __syncthreads();
  auto load_plane = [&](int kk, bool phi_only) {  // thread 0
    uint64_t *bar = &bars[kk & 3];
    if (kk >= 0 && kk < PZ) {
      mbar_expect_tx(bar, (unsigned)(sizeof(float) * (kQPhiPL + (phi_only ? 0 : 4 * kQPL))));
      if (!phi_only)
#pragma unroll
        for (int f = 0; f < 4; ++f) tma_load_3d(&ring.f[f][kk & 3][0], &maps.m[f], i0 - 5, j0 - 1, kk, bar);
      tma_load_3d(&ring.phi[kk & 3][0], &maps.m[4], i0 - 5, j0 - 2, kk, bar);
    } else {
      mbar_arrive(bar);
    }
  };
  bool tma_ok = true;
  auto wait_plane = [&](int kk) {
    if (tma_ok && !mbar_wait(&bars[kk & 3], ((kk - kfirst) >> 2) & 1)) {
      tma_ok = false;
      if (kerr) atomicExch(kerr, 1);
    }
  };
  const int i = i0 + 2 * tx, j = j0 + ty;  // the pair (i, i + 1)
  // the other set's values at the pair and the stored residuals of the
  // input state, prefetched one plane ahead (single elements: the pair
  // starts at an odd index)
  const bool in_a = i < PX && j < g.PY, in_b = i + 1 < PX && j < g.PY;
  const long qij = (long)i + PX * (long)j;
  const float *const oth0 = F.vel(oth_set, 0) + qij, *const oth1 = F.vel(oth_set, 1) + qij,
                     *const oth2 = F.vel(oth_set, 2) + qij;
  const __nv_bfloat16 *const res0 = res.c[0] + qij, *const res1 = res.c[1] + qij, *const res2 = res.c[2] + qij;
  float2 n0 = splat2(0.f), n1 = n0, n2 = n0, l0 = n0, l1 = n0, l2 = n0;
  auto prefetch = [&](int kk) {
    if (kk >= kend) return;
    const long po = (long)kk * plane;
    if (in_a) {
      if (kOth) n0.x = oth0[po], n1.x = oth1[po], n2.x = oth2[po];
      l0.x = __bfloat162float(res0[po]), l1.x = __bfloat162float(res1[po]), l2.x = __bfloat162float(res2[po]);
    }
    if (in_b) {
      if (kOth) n0.y = oth0[po + 1], n1.y = oth1[po + 1], n2.y = oth2[po + 1];
      l0.y = __bfloat162float(res0[po + 1]), l1.y = __bfloat162float(res1[po + 1]),
      l2.y = __bfloat162float(res2[po + 1]);
    }
  };
  // Interior masks in x and y, bit c + 3 s for component c at point s: the
  // own pair (s = 0, 1) and this thread's halo pair or point (s = 2, 3).
  auto xy_mask = [&](int x, int y) {
    unsigned m = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      if (x >= 1 && y >= 1 && x < g.ext(c, 0) - 1 && y < g.ext(c, 1) - 1) m |= 1u << c;
    return m;
  };
  const bool h_pair = tid < 2 * kTX, h_single = tid >= 2 * kTX && tid < 2 * kTX + kQHaloCols;
  int h_r = 0, h_p = 0;
  unsigned msk = xy_mask(i, j) | (xy_mask(i + 1, j) << 3);
  {
    int hx = 0, hy = 0;
    if (tid < kTX) hx = 5 + 2 * tid, hy = 0;
    else if (tid < 2 * kTX) hx = 5 + 2 * (tid - kTX), hy = kTY + 1;
    else if (tid < 2 * kTX + kTY + 2) hx = 4, hy = tid - 2 * kTX;
    else hx = kQX + 5, hy = tid - 2 * kTX - (kTY + 2);
    h_r = hy * kQHX + hx;
    h_p = (hy + 1) * kQHX + hx;
    const int hi_ = i0 - 5 + hx, hj = j0 - 1 + hy;
    if (h_pair) msk |= (xy_mask(hi_, hj) << 6) | (xy_mask(hi_ + 1, hj) << 9);
    if (h_single) msk |= xy_mask(hi_, hj) << 6;
  }
  const int o_r = (ty + 1) * kQHX + 5 + 2 * tx, o_p = o_r + kQHX;  // own ring / phi index (odd)
  float2 e0 = splat2(0.f), e1 = e0, e2 = e0;  // the own pair's exact residuals at the plane projected last
  // Projection of ring plane kk (u' = fl(u + inc), inc = (phi_b - phi) oh dt,
  // on the points interior to the component); with own_exact the own pair's
  // stored residuals lo become lo + e (e0..e2). (Adding the stored residual
  // one plane later instead, so that its load had a plane of work to land,
  // kept six more registers live; the spills cost more than the wait.)
  auto project_plane = [&](int kk, bool own_exact) {
    float *const rb = ring.f[0][kk & 3];
    const float *const ph = ring.phi[kk & 3], *const phb = ring.phi[(kk - 1) & 3];
    const unsigned kin = (kk >= 1) ? ((kk < lim0 ? 1u : 0u) | (kk < lim1 ? 2u : 0u) | (kk < lim2 ? 4u : 0u)) : 0u;
    const unsigned m = msk & (kin * 0x249u);  // kin in every point's bits
    {
      const float2 fm = lda2(ph, o_p - 1), fp = lda2(ph, o_p + 1), f0 = make_float2(fm.y, fp.x);
      float2 lo[3] = {l0, l1, l2};
      const float2 fb[3] = {fm, ldp2(ph, o_p - kQHX), ldp2(phb, o_p)};
      const float2 cd[3] = {cd0, cd1, cd2};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const bool ma = (m >> c) & 1u, mb = (m >> (3 + c)) & 1u;
        if (!(ma || mb)) continue;
        float *const r = rb + c * 4 * kQSlot + o_r;
        const float2 hi = make_float2(r[0], r[1]);
        const float2 inc = mul2(sub2(fb[c], f0), cd[c]);
        const float2 s = add2(hi, inc);
        const float2 e = two_sum_err2(hi, inc, s);
        if (ma) r[0] = s.x, lo[c].x = __fadd_rn(lo[c].x, e.x);
        if (mb) r[1] = s.y, lo[c].y = __fadd_rn(lo[c].y, e.y);
      }
      if (own_exact) e0 = lo[0], e1 = lo[1], e2 = lo[2];
    }
    if (h_pair && (m & 0xfc0u)) {
      const float2 fm = lda2(ph, h_p - 1), fp = lda2(ph, h_p + 1), f0 = make_float2(fm.y, fp.x);
      const float2 fb[3] = {fm, ldp2(ph, h_p - kQHX), ldp2(phb, h_p)};
      const float2 cd[3] = {cd0, cd1, cd2};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const bool ma = (m >> (6 + c)) & 1u, mb = (m >> (9 + c)) & 1u;
        if (!(ma || mb)) continue;
        float *const r = rb + c * 4 * kQSlot + h_r;
        const float2 s = add2(make_float2(r[0], r[1]), mul2(sub2(fb[c], f0), cd[c]));
        if (ma) r[0] = s.x;
        if (mb) r[1] = s.y;
      }
    } else if (h_single && (m & 0x1c0u)) {
      const float f0 = ph[h_p];
      if (m & 0x40u) rb[h_r] = __fadd_rn(rb[h_r], (ph[h_p - 1] - f0) * cd0.x);
      if (m & 0x80u) rb[4 * kQSlot + h_r] = __fadd_rn(rb[4 * kQSlot + h_r], (ph[h_p - kQHX] - f0) * cd1.x);
      if (m & 0x100u) rb[8 * kQSlot + h_r] = __fadd_rn(rb[8 * kQSlot + h_r], (phb[h_p] - f0) * cd2.x);
    }
  };
  // p + phi, stochastically rounded: the pair's two dithers from one hash.
  const unsigned psalt = sr_salt(tr, pj.tag);
  auto p_new1 = [&](int r, int rp, int kk, long q) {
    return add_sr(ring.f[3][kk & 3][r], ring.phi[kk & 3][rp], sr_draw(sr_mix((unsigned)q ^ psalt), 0));
  };
  // Pressure nodes outside the threads' range, at the CTAs on those edges.
  const int E0 = g.E[0], E1 = g.E[1], E2 = g.E[2];
  // the last node E0 - 1 is the right halo only of the last tile (else a
  // later tile owns it)
  const bool edge_x0 = blockIdx.x == 0, edge_y0 = blockIdx.y == 0,
             edge_xr = i0 + kQX == E0 - 1 && blockIdx.x + 1 == gridDim.x;
  auto write_p_edges = [&](int kk) {
    auto one = [&](int hx, int hy) {
      const int pi = i0 - 5 + hx, pjj = j0 - 1 + hy;
      if (pi >= E0 || pjj >= E1 || kk >= E2) return;
      const long q = pi + PX * (pjj + g.PY * (long)kk);
      p_out[q] = p_new1(hy * kQHX + hx, (hy + 1) * kQHX + hx, kk, q);
    };
    if (edge_x0 && tx == 0) one(4, ty + 1);
    if (edge_xr && tx == kTX - 1) one(kQX + 5, ty + 1);
    if (edge_y0 && ty == 0) {
      one(5 + 2 * tx, 0);
      one(6 + 2 * tx, 0);
      if (edge_x0 && tx == 0) one(4, 0);
      if (edge_xr && tx == kTX - 1) one(kQX + 5, 0);
    }
  };
  const bool own_pa = i < E0 && j < E1, own_pb = i + 1 < E0 && j < E1;
  auto write_p_pair = [&](int kk, long q) {
    const float2 pv = ldp2(ring.f[3][kk & 3], o_r), fv = ldp2(ring.phi[kk & 3], o_p);
    const unsigned h = sr_mix((unsigned)q ^ psalt);
    const float2 s = add_sr2(pv, fv, make_float2(sr_draw(h, 0), sr_draw(h, 1)));
    if (own_pa) p_out[q] = s.x;
    if (own_pb) p_out[q + 1] = s.y;
  };
  const bool edges = edge_x0 | edge_y0 | edge_xr;
  // Prologue: phi of plane kbeg - 2 (w's projection of plane kbeg - 1), the
  // planes kbeg - 1 .. kbeg + 1; planes kbeg - 1 and kbeg projected.
  if (tid == 0) {
    load_plane(kbeg - 2, true);
    load_plane(kbeg - 1, false);
    load_plane(kbeg, false);
    load_plane(kbeg + 1, false);
  }
  wait_plane(kbeg - 2);
  wait_plane(kbeg - 1);
  wait_plane(kbeg);
  project_plane(kbeg - 1, false);
  prefetch(kbeg);
  project_plane(kbeg, true);
  if (kbeg == 1) {  // the pressure of plane 0, which no thread's march reaches
    write_p_pair(0, qij);
    if (edges) write_p_edges(0);
  }
  __syncthreads();  // the first iteration refills the slot of plane kbeg - 2
  for (int k = kbeg; k < kend; ++k) {
    if (tid == 0 && k + 2 <= kend) {
      fence_async_shared();
      load_plane(k + 2, false);
    }
    const float2 c0 = n0, c1 = n1, c2 = n2, lo0 = e0, lo1 = e1, lo2 = e2;
    prefetch(k + 1);
    wait_plane(k + 1);
    project_plane(k + 1, true);
    __syncthreads();
    const float *U[3], *V[3], *W[3], *P[3];
#pragma unroll
    for (int dk = -1; dk <= 1; ++dk) {
      U[dk + 1] = ring.f[0][(k + dk) & 3];
      V[dk + 1] = ring.f[1][(k + dk) & 3];
      W[dk + 1] = ring.f[2][(k + dk) & 3];
      P[dk + 1] = ring.f[3][(k + dk) & 3];
    }
    const float *const ph = ring.phi[k & 3], *const phb = ring.phi[(k - 1) & 3];
    const float2 fm = lda2(ph, o_p - 1), fp = lda2(ph, o_p + 1), f14 = make_float2(fm.y, fp.x);
    const long q = qij + (long)k * plane;
    auto update = [&](auto cc, const float2 &cur, const float2 &lo, float2 fb, float ohc) {
      constexpr int c = decltype(cc)::value;
      const bool ma = (msk >> c) & 1u, mb = (msk >> (3 + c)) & 1u;
      if (!(ma || mb) || k >= (c == 0 ? lim0 : (c == 1 ? lim1 : lim2))) return;
      float2 self, dp;
      const float2 r = rhs_pair<c>(U, V, W, P, o_r, co, self, dp);
      const float2 gp = mul2(add2(dp, sub2(f14, fb)), splat2(ohc));
      float2 inc, err, s;
      float *const out_s = F.vel(ST == kStageY2 ? 1 : (ST == kStageY3 ? 2 : 0), c) + q;
      if constexpr (ST == kStageY2) {
        inc = fma2(splat2(-K.k3), gp, mul2(splat2(K.k1), r));
      } else if constexpr (ST == kStageY3) {
        const float2 r2s = mul2(splat2(K.k2), r);
        inc = fma2(splat2(-K.k3), gp, fma2(splat2(K.k1), cur, r2s));
        float *const out_r = F.vel(0, c) + q;
        if (ma) out_r[0] = r2s.x;
        if (mb) out_r[1] = r2s.y;
      } else {
        inc = sub2(fma2(splat2(-K.k3), gp, mul2(splat2(K.k2), r)), cur);
      }
      s = comp_add2(self, lo, inc, err);
      __nv_bfloat16 *const lo_out = res.c[c] + q;
      if (ma) out_s[0] = s.x, lo_out[0] = __float2bfloat16_rn(err.x);
      if (mb) out_s[1] = s.y, lo_out[1] = __float2bfloat16_rn(err.y);
      if constexpr (ST == kStageY2) {
        float *const out_r = F.vel(2, c) + q;
        if (ma) out_r[0] = r.x;
        if (mb) out_r[1] = r.y;
      }
    };
    update(std::integral_constant<int, 0>{}, c0, lo0, fm, oh0);
    update(std::integral_constant<int, 1>{}, c1, lo1, ldp2(ph, o_p - kQHX), oh1);
    update(std::integral_constant<int, 2>{}, c2, lo2, ldp2(phb, o_p), oh2);
    write_p_pair(k, q);
    if (edges) write_p_edges(k);
    __syncthreads();  // the next iteration refills the slot of plane k - 1
  }
}

// ---- boundary fill, src/VelocityTensor.cpp:36-233 ----

// Sampling point of component c at index (i,j,k): staggered (face) along c.
__device__ __forceinline__ void stag_point(const Geometry &g, int c, const long *ix, double *x) {
#pragma unroll
  for (int d = 0; d < 3; ++d) x[d] = d == c ? g.face(d, ix[d]) : g.node(d, ix[d]);
}

// Value the reference writes at a Dirichlet face point of component c whose
// winning face is axis d, side s (0 min, 1 max).
template <typename TE>
__device__ TE face_value(const Geometry &g, int c, int d, int s, const long *pt, int kind, int fn, TE t) {
  const TE Re = TE(g.Re);
  if (c != d) {
    double x[3];
    stag_point(g, c, pt, x);
    return analytic_vector<TE>(fn, kind, c, t, TE(x[0]), TE(x[1]), TE(x[2]), Re);
  }
  // Normal component: boundary value at the node plus h/2 times the exact
  // tangential divergence (src/VelocityTensor.cpp:47-61,163-207).
  long q[3] = {pt[0], pt[1], pt[2]};
  q[d] = s == 0 ? 0 : g.E[d] - 1;
  const TE xb = TE(g.node(0, q[0])), yb = TE(g.node(1, q[1])), zb = TE(g.node(2, q[2]));
  const TE base = analytic_vector<TE>(fn, kind, c, t, xb, yb, zb, Re);
  TE sum = TE(0);
  bool first = true;
#pragma unroll
  for (int c2 = 0; c2 < 3; ++c2) {
    if (c2 == d) continue;
    long q1[3] = {q[0], q[1], q[2]};
    q1[c2] += 1;
    double x0[3], x1[3];
    stag_point(g, c2, q1, x1);
    stag_point(g, c2, q, x0);
    const TE f1 = analytic_vector<TE>(fn, kind, c2, t, TE(x1[0]), TE(x1[1]), TE(x1[2]), Re);
    const TE f0 = analytic_vector<TE>(fn, kind, c2, t, TE(x0[0]), TE(x0[1]), TE(x0[2]), Re);
    const TE der = (f1 - f0) * TE(g.oh[c2]);
    sum = first ? der : sum + der;
    first = false;
  }
  return s == 0 ? base + TE(g.h_2[d]) * sum : base - TE(g.h_2[d]) * sum;
}

// blockIdx.z = d: faces normal to axis d; one thread takes face point
// (pa, pb) of all three components, both sides. Each face point is written
// once, by the face the reference writes last (order z_min, z_max, y_min,
// y_max, x_min, x_max). kTable: the values come from the double face tables
// only (ft.tab set), so the analytic families' code, and the registers it
// needs, are left out of that instantiation.
template <typename T, bool kTable>
__global__ void bc_faces_kernel(Geometry g, T *c0, T *c1, T *c2, int kind, int fn, TimeRef tr, int t_slot,
                                FaceTables ft, Residual res) {
  const int d = blockIdx.z;
  if (g.periodic[d]) return;
  const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
  const long pa = blockIdx.x * blockDim.x + threadIdx.x;
  const long pb = blockIdx.y * blockDim.y + threadIdx.y;
  if (pa >= g.Es[a] || pb >= g.Es[b]) return;  // the widest extents of the three components
  const double t = tr.get(t_slot);
  // caller data (slot_stride > 0): the slot's own table, no time factor
  const double factor = ft.tab ? (ft.slot_stride ? 1.0 : tr.get(kSlotFactor + 4 * fn + t_slot)) : 0.0;
  const double *tab = ft.tab ? ft.tab + (long)t_slot * ft.slot_stride : nullptr;
  if constexpr (kTable) {
    // From the tables: the six face values (three components, both sides)
    // are all loaded before any is stored, so their loads overlap (the
    // compiler cannot move a table load above a field store).
    double v[3][2];
    long q[3][2];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        q[c][s] = -1;
        if (pa >= g.ext(c, a) || pb >= g.ext(c, b)) continue;
        const long fixed = s == 0 ? 0 : g.ext(c, d) - 1;
        const long pt[3] = {d == 0 ? fixed : pa, d == 1 ? fixed : (d == 0 ? pa : pb), d == 2 ? fixed : pb};
        bool later = false;  // an x face beats y beats z
        if (d >= 1 && !g.periodic[0] && (pt[0] == 0 || pt[0] == g.ext(c, 0) - 1)) later = true;
        if (d == 2 && !g.periodic[1] && (pt[1] == 0 || pt[1] == g.ext(c, 1) - 1)) later = true;
        if (later) continue;
        q[c][s] = g.idx(pt[0], pt[1], pt[2]);
        v[c][s] = __ldg(tab + ft.off[fn][c][d][s] + pa + (long)g.ext(c, a) * pb) * factor;
      }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T *f = c == 0 ? c0 : (c == 1 ? c1 : c2);
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        if (q[c][s] < 0) continue;
        if constexpr (std::is_same<T, float>::value) {
          if (res.on()) {  // compensated state: the double face value as hi + residual
            f[q[c][s]] = comp_split(v[c][s], res.c[c] + q[c][s]);
            continue;
          }
        }
        f[q[c][s]] = T(v[c][s]);
      }
    }
    return;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (pa >= g.ext(c, a) || pb >= g.ext(c, b)) continue;
    T *f = c == 0 ? c0 : (c == 1 ? c1 : c2);
    for (int s = 0; s < 2; ++s) {
      // the point's (x, y, z): the face's fixed coordinate along d, pa and pb
      // along the other two axes in order
      const long fixed = s == 0 ? 0 : g.ext(c, d) - 1;
      const long pt[3] = {d == 0 ? fixed : pa, d == 1 ? fixed : (d == 0 ? pa : pb), d == 2 ? fixed : pb};
      bool later = false;  // an x face beats y beats z
      if (d >= 1 && !g.periodic[0] && (pt[0] == 0 || pt[0] == g.ext(c, 0) - 1)) later = true;
      if (d == 2 && !g.periodic[1] && (pt[1] == 0 || pt[1] == g.ext(c, 1) - 1)) later = true;
      if (later) continue;
      // evaluated in the working precision (no tables)
      const long q = g.idx(pt[0], pt[1], pt[2]);
      if constexpr (std::is_same<T, float>::value) {
        if (res.on()) {  // compensated state: the value as hi + residual
          f[q] = comp_split((double)face_value<T>(g, c, d, s, pt, kind, fn, T(t)), res.c[c] + q);
          continue;
        }
      }
      f[q] = T(face_value<T>(g, c, d, s, pt, kind, fn, T(t)));
    }
  }
}

// Periodic copies of all axes at once (src/StaggeredTensor.cpp:221-257).
// Along x, then y, then z the reference copies a[0] = a[E-2], a[E-1] = a[1]
// over the whole face, ghosts of the other axes included; composed, every
// ghost point ends equal to its image Q (each ghost coordinate 0 -> E-2,
// E-1 -> 1), a non-ghost point, whatever the order. One thread per ghost
// point copies f[Q] (reads non-ghost, writes ghost: no conflicts), so the
// result is bitwise the three passes'. blockIdx.z = comp * 6 + face: the
// ghost plane 0 / E-1 of periodic axis d, a point counted only on its first
// ghost axis.
template <typename T>
__global__ void periodic_kernel(Geometry g, T *f0, T *f1, T *f2, int scalar, Residual res) {
  const int c = blockIdx.z / 6, face = blockIdx.z % 6, d = face / 2, side = face % 2;
  T *f = c == 0 ? f0 : (c == 1 ? f1 : f2);
  if (!f || !g.periodic[d]) return;
  int ex[3];
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) ex[ax] = scalar ? g.E[ax] : g.ext(c, ax);
  const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
  const int pa = blockIdx.x * blockDim.x + threadIdx.x, pb = blockIdx.y * blockDim.y + threadIdx.y;
  if (pa >= ex[a] || pb >= ex[b]) return;
  int p[3];
  p[d] = side == 0 ? 0 : ex[d] - 1;
  p[a] = pa;
  p[b] = pb;
  int q[3];
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    const bool ghost = g.periodic[ax] && (p[ax] == 0 || p[ax] == ex[ax] - 1);
    if (ghost && ax < d) return;  // counted on an earlier axis's ghost plane
    q[ax] = !ghost ? p[ax] : (p[ax] == 0 ? ex[ax] - 2 : 1);
  }
  const long dst = g.idx(p[0], p[1], p[2]), src = g.idx(q[0], q[1], q[2]);
  f[dst] = f[src];
  if (res.on() && !scalar) res.c[c][dst] = res.c[c][src];
}

// ---- Poisson right-hand side and projection ----

// Each thread owns KZ consecutive owner planes of one (i, j) column; the
// loads of all its points are issued before any result is stored.
constexpr int kDivKZ = 4;
// The compensated divergence (divergence_pair_kernel) reads five more
// values per point, the residuals: two planes per thread keep its register
// count near the plain kernel's.
constexpr int kDivKZComp = 2;

template <typename T, int KZ = kDivKZ>
__global__ void __launch_bounds__(128) divergence_kernel(Geometry g, T *__restrict__ phi, const T *__restrict__ u,
                                                         const T *__restrict__ v, const T *__restrict__ w, T inv_dt) {
  const int i = g.own_lo[0] + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.own_lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
  const int kb = g.own_lo[2] + blockIdx.z * KZ;
  const int ke = min(kb + KZ, g.own_lo[2] + g.np[2]);
  if (i >= g.own_lo[0] + g.np[0] || j >= g.own_lo[1] + g.np[1]) return;
  const long q0 = g.idx(i, j, kb), sy = g.sy(), sz = g.sz();
  T a[KZ], b[KZ], c[KZ], d[KZ], e[KZ + 1];
  e[0] = ld(w, q0);
#pragma unroll
  for (int r = 0; r < KZ; ++r) {
    if (kb + r >= ke) break;
    const long q = q0 + r * sz;
    a[r] = ld(u, q + 1);
    b[r] = ld(u, q);
    c[r] = ld(v, q + sy);
    d[r] = ld(v, q);
    e[r + 1] = ld(w, q + sz);
  }
#pragma unroll
  for (int r = 0; r < KZ; ++r) {
    if (kb + r >= ke) break;
    const T du = (a[r] - b[r]) * T(g.oh[0]);
    const T dv = (c[r] - d[r]) * T(g.oh[1]);
    const T dw = (e[r + 1] - e[r]) * T(g.oh[2]);
    phi[q0 + r * sz] = (du + dv + dw) * inv_dt;
  }
}

// The compensated divergence: the velocity is hi + residual, and each
// difference adds the residuals' difference, so the float divergence sees
// the compensated state: ((a - b) + (la - lb)) / h per axis, summed as in
// divergence_kernel. Two adjacent x points per thread: the velocity in
// aligned 8-byte float pairs and the residuals in 4-byte bfloat16 pairs (a
// pair starts at an even x and PX is even). Pairs run over x from 0; a point
// outside the owner range is read but not written.
template <int KZ>
__global__ void __launch_bounds__(128)
    divergence_pair_kernel(Geometry g, float *__restrict__ phi, const float *__restrict__ u,
                           const float *__restrict__ v, const float *__restrict__ w, float inv_dt, Residual res) {
  const int i0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int j = g.own_lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
  const int kb = g.own_lo[2] + blockIdx.z * KZ;
  const int ke = min(kb + KZ, g.own_lo[2] + g.np[2]);
  const int x_lo = g.own_lo[0], x_hi = g.own_lo[0] + g.np[0];
  const bool ok0 = i0 >= x_lo && i0 < x_hi, ok1 = i0 + 1 >= x_lo && i0 + 1 < x_hi;
  if ((!ok0 && !ok1) || j >= g.own_lo[1] + g.np[1]) return;
  const long q0 = g.idx(i0, j, kb), sy = g.sy(), sz = g.sz();
  auto f2 = [](const float *f, long q) { return __ldg(reinterpret_cast<const float2 *>(f + q)); };
  auto b2 = [](const __nv_bfloat16 *f, long q) {
    return __bfloat1622float2(__ldg(reinterpret_cast<const __nv_bfloat162 *>(f + q)));
  };
  float2 ua[KZ], va[KZ], vb[KZ], we[KZ + 1], lua[KZ], lva[KZ], lvb[KZ], lwe[KZ + 1];
  float u2[KZ], lu2[KZ];
  we[0] = f2(w, q0);
  lwe[0] = b2(res.c[2], q0);
#pragma unroll
  for (int r = 0; r < KZ; ++r) {
    if (kb + r >= ke) break;
    const long q = q0 + r * sz;
    ua[r] = f2(u, q);
    va[r] = f2(v, q);
    vb[r] = f2(v, q + sy);
    we[r + 1] = f2(w, q + sz);
    lua[r] = b2(res.c[0], q);
    lva[r] = b2(res.c[1], q);
    lvb[r] = b2(res.c[1], q + sy);
    lwe[r + 1] = b2(res.c[2], q + sz);
    // u one point past the pair, for its second point
    u2[r] = ok1 ? __ldg(u + q + 2) : 0.f;
    lu2[r] = ok1 ? __bfloat162float(__ldg(res.c[0] + q + 2)) : 0.f;
  }
  const float oh0 = float(g.oh[0]), oh1 = float(g.oh[1]), oh2 = float(g.oh[2]);
#pragma unroll
  for (int r = 0; r < KZ; ++r) {
    if (kb + r >= ke) break;
    float du = ua[r].y - ua[r].x, dv = vb[r].x - va[r].x, dw = we[r + 1].x - we[r].x;
    du += lua[r].y - lua[r].x;
    dv += lvb[r].x - lva[r].x;
    dw += lwe[r + 1].x - lwe[r].x;
    du = du * oh0;
    dv = dv * oh1;
    dw = dw * oh2;
    float2 out;
    out.x = (du + dv + dw) * inv_dt;
    du = u2[r] - ua[r].y;
    dv = vb[r].y - va[r].y;
    dw = we[r + 1].y - we[r].y;
    du += lu2[r] - lua[r].y;
    dv += lvb[r].y - lva[r].y;
    dw += lwe[r + 1].y - lwe[r].y;
    du = du * oh0;
    dv = dv * oh1;
    dw = dw * oh2;
    out.y = (du + dv + dw) * inv_dt;
    const long q = q0 + r * sz;
    if (ok0 && ok1) {
      *reinterpret_cast<float2 *>(phi + q) = out;
    } else if (ok0) {
      phi[q] = out.x;
    } else {
      phi[q + 1] = out.y;
    }
  }
}

template <typename T>
__global__ void neumann_flux_serial_kernel(Geometry g, T *phi, int kind, TimeRef tr, int slot_new, int slot_old) {
  const double t_new = tr.get(slot_new), t_old = tr.get(slot_old);
  // Every boundary node is visited by one thread, which adds the terms of all
  // faces containing it in the reference's order (z, then y, then x).
  const long n_total = (long)g.E[0] * g.E[1] * g.E[2];
  const long id = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= n_total) return;
  const long i = id % g.E[0], j = (id / g.E[0]) % g.E[1], k = id / ((long)g.E[0] * g.E[1]);
  const bool onb = i == 0 || i == g.E[0] - 1 || j == 0 || j == g.E[1] - 1 || k == 0 || k == g.E[2] - 1;
  if (!onb) return;
  const double x = g.node(0, i), y = g.node(1, j), z = g.node(2, k);
  auto G = [&](int c) {
    return T(analytic_pressure_gradient<T>(kind, c, T(t_old), T(x), T(y), T(z), T(g.Re)) -
             analytic_pressure_gradient<T>(kind, c, T(t_new), T(x), T(y), T(z), T(g.Re)));
  };
  const long q = g.idx(i, j, k);
  T r = phi[q];
  if (k == 0) r += G(2) * T(2.0) * T(g.oh[2]);
  if (k == g.E[2] - 1) r -= G(2) * T(2.0) * T(g.oh[2]);
  if (j == 0) r += G(1) * T(2.0) * T(g.oh[1]);
  if (j == g.E[1] - 1) r -= G(1) * T(2.0) * T(g.oh[1]);
  if (i == 0) r += G(0) * T(2.0) * T(g.oh[0]);
  if (i == g.E[0] - 1) r -= G(0) * T(2.0) * T(g.oh[0]);
  phi[q] = r;
}

// Boundary nodes from caller data. blockIdx.z = f, the face (x_min, x_max,
// y_min, y_max, z_min, z_max) whose threads own its nodes; a node on several
// faces belongs to the first of them in that order, and its one thread adds
// the terms of all its faces in the reference's order (z, then y, then x
// faces, each min before max), so every node is written once.
template <typename T>
__global__ void neumann_flux_data_kernel(Geometry g, T *phi, const double *G, GradFaces gf) {
  const int f = blockIdx.z, d = f / 2, side = f % 2;
  const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
  const long pa = blockIdx.x * blockDim.x + threadIdx.x, pb = blockIdx.y * blockDim.y + threadIdx.y;
  if (pa >= g.E[a] || pb >= g.E[b]) return;
  long p[3];
  p[d] = side ? g.E[d] - 1 : 0;
  p[a] = pa;
  p[b] = pb;
  for (int d2 = 0; d2 < d; ++d2)
    if (p[d2] == 0 || p[d2] == g.E[d2] - 1) return;  // owned by an x (or y) face
  if (side == 1 && p[d] == 0) return;
  const long i = p[0], j = p[1], k = p[2];
  const long E0 = g.E[0], E1 = g.E[1];
  const long q = g.idx(i, j, k);
  T r = phi[q];
  if (k == 0) r += T(G[gf.off[4] + i + E0 * j]) * T(2.0) * T(g.oh[2]);
  if (k == g.E[2] - 1) r -= T(G[gf.off[5] + i + E0 * j]) * T(2.0) * T(g.oh[2]);
  if (j == 0) r += T(G[gf.off[2] + i + E0 * k]) * T(2.0) * T(g.oh[1]);
  if (j == g.E[1] - 1) r -= T(G[gf.off[3] + i + E0 * k]) * T(2.0) * T(g.oh[1]);
  if (i == 0) r += T(G[gf.off[0] + j + E1 * k]) * T(2.0) * T(g.oh[0]);
  if (i == g.E[0] - 1) r -= T(G[gf.off[1] + j + E1 * k]) * T(2.0) * T(g.oh[0]);
  phi[q] = r;
}

// Each thread owns kProjKZ consecutive planes of one (i, j) column. Two
// planes keep it at 32 registers (full occupancy); on GB300 at 512^3 the
// projection measured 2.76 / 2.44 / 2.77 / 3.13 ms per step for 1 / 2 / 4 / 8.
constexpr int kProjKZ = 2;

// nonfinite (may be null): set to 1 when a phi value read is NaN or Inf. A
// NaN or Inf anywhere in the velocity reaches every phi value through the
// divergence and the spectral solve, so this one check per point watches
// the whole step.
template <typename T>
__global__ void __launch_bounds__(128) project_kernel(Geometry g, T *__restrict__ p, const T *__restrict__ phi,
                                                      T *__restrict__ u, T *__restrict__ v, T *__restrict__ w, T dt,
                                                      TimeRef tr, unsigned tag, int *nonfinite) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int kb = blockIdx.z * kProjKZ;
  const long sy = g.sy(), sz = g.sz();
  T *vel[3] = {u, v, w};
  const long sc[3] = {1, sy, sz};
  T ph[kProjKZ + 1], nb[2][kProjKZ], pv[kProjKZ], vv[3][kProjKZ];
  // loads: phi at the points, their -x and -y neighbours, the plane below, p and the velocity
  ph[0] = (kb >= 1 && i < g.E[0] && j < g.E[1] && kb - 1 < g.E[2]) ? ld(phi, g.idx(i, j, kb - 1)) : T(0);
#pragma unroll
  for (int r = 0; r < kProjKZ; ++r) {
    const int k = kb + r;
    const long q = g.idx(i, j, k);
    const bool inp = i < g.E[0] && j < g.E[1] && k < g.E[2];
    ph[r + 1] = inp ? ld(phi, q) : T(0);
    nb[0][r] = (inp && i >= 1) ? ld(phi, q - 1) : T(0);
    nb[1][r] = (inp && j >= 1) ? ld(phi, q - sy) : T(0);
    pv[r] = inp ? p[q] : T(0);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const bool in = i >= 1 && j >= 1 && k >= 1 && i < g.ext(c, 0) - 1 && j < g.ext(c, 1) - 1 && k < g.ext(c, 2) - 1;
      vv[c][r] = in ? vel[c][q] : T(0);
    }
  }
  constexpr bool kSR = std::is_same<T, float>::value;
  const unsigned salt = kSR ? sr_salt(tr, tag) : 0u;
  if (nonfinite) {
    bool bad = false;
#pragma unroll
    for (int r = 0; r <= kProjKZ; ++r) bad |= !isfinite(ph[r]);
    if (bad) *nonfinite = 1;
  }
#pragma unroll
  for (int r = 0; r < kProjKZ; ++r) {
    const int k = kb + r;
    const long q = g.idx(i, j, k);
    const unsigned h = kSR ? sr_mix((unsigned)q ^ salt) : 0u;
    const unsigned h2 = kSR ? sr_mix(h) : 0u;
    if (i < g.E[0] && j < g.E[1] && k < g.E[2])
      p[q] = kSR ? state_add(pv[r], ph[r + 1], sr_draw(h2, 0)) : pv[r] + ph[r + 1];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (i < 1 || j < 1 || k < 1 || i >= g.ext(c, 0) - 1 || j >= g.ext(c, 1) - 1 || k >= g.ext(c, 2) - 1) continue;
      const T below = c == 0 ? nb[0][r] : (c == 1 ? nb[1][r] : ph[r]);
      const T gp = (ph[r + 1] - below) * T(g.oh[c]);
      vel[c][q] = kSR ? state_add(vv[c][r], -(gp * dt), sr_draw(h, c)) : vv[c][r] - gp * dt;
    }
  }
  (void)sc;
}

// The compensated projection: the masks, the gradient and the pressure's
// stochastically rounded update of project_kernel, with the velocity update
// an error-free sum into hi + residual (comp_add). Two adjacent x points and
// one plane per thread: phi, p, the velocity and the residuals in aligned
// pairs (8-byte floats, 4-byte bfloat16 pairs). A pair whose two points need
// different updates stores them one by one.
__global__ void __launch_bounds__(128)
    project_pair_kernel(Geometry g, float *__restrict__ p, const float *__restrict__ phi, float *__restrict__ u,
                        float *__restrict__ v, float *__restrict__ w, float dt, TimeRef tr, unsigned tag,
                        Residual res, int *nonfinite) {
  const int i0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i0 >= g.PX || j >= g.PY) return;
  const long sy = g.sy(), sz = g.sz();
  const long q = g.idx(i0, j, k);
  float *vel[3] = {u, v, w};
  auto f2 = [](const float *f, long qq) { return *reinterpret_cast<const float2 *>(f + qq); };
  const bool jk_in = j < g.E[1] && k < g.E[2];
  const bool inp[2] = {jk_in && i0 < g.E[0], jk_in && i0 + 1 < g.E[0]};
  float2 ph = make_float2(0.f, 0.f), below_z = make_float2(0.f, 0.f), below_y = make_float2(0.f, 0.f);
  float below_x0 = 0.f, pv[2] = {0.f, 0.f};
  if (inp[0] || inp[1]) {
    const float2 a = __ldg(reinterpret_cast<const float2 *>(phi + q));
    ph = make_float2(inp[0] ? a.x : 0.f, inp[1] ? a.y : 0.f);
    if (k >= 1) {
      const float2 b = __ldg(reinterpret_cast<const float2 *>(phi + q - sz));
      below_z = make_float2(inp[0] ? b.x : 0.f, inp[1] ? b.y : 0.f);
    }
    if (j >= 1) {
      const float2 b = __ldg(reinterpret_cast<const float2 *>(phi + q - sy));
      below_y = make_float2(inp[0] ? b.x : 0.f, inp[1] ? b.y : 0.f);
    }
    if (inp[0] && i0 >= 1) below_x0 = __ldg(phi + q - 1);
    const float2 pp = f2(p, q);
    pv[0] = pp.x;
    pv[1] = pp.y;
  }
  // interior of component c at the two points, their values and residuals
  bool in[3][2];
  float2 vv[3], lv[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const bool jk = j >= 1 && k >= 1 && j < g.ext(c, 1) - 1 && k < g.ext(c, 2) - 1;
    in[c][0] = jk && i0 >= 1 && i0 < g.ext(c, 0) - 1;
    in[c][1] = jk && i0 + 1 < g.ext(c, 0) - 1;
    vv[c] = make_float2(0.f, 0.f);
    lv[c] = make_float2(0.f, 0.f);
    if (in[c][0] || in[c][1]) {
      vv[c] = f2(vel[c], q);
      lv[c] = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(res.c[c] + q));
    }
  }
  if (nonfinite && !(isfinite(ph.x) && isfinite(ph.y) && isfinite(below_z.x) && isfinite(below_z.y)))
    *nonfinite = 1;
  const unsigned salt = sr_salt(tr, tag);
  float pout[2];
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const float phe = e ? ph.y : ph.x;
    const unsigned h = sr_mix((unsigned)(q + e) ^ salt);
    pout[e] = state_add(pv[e], phe, sr_draw(sr_mix(h), 0));
  }
  if (inp[0] && inp[1])
    *reinterpret_cast<float2 *>(p + q) = make_float2(pout[0], pout[1]);
  else if (inp[0])
    p[q] = pout[0];
  else if (inp[1])
    p[q + 1] = pout[1];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (!in[c][0] && !in[c][1]) continue;
    float out[2];
    __nv_bfloat16 lo[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const float phe = e ? ph.y : ph.x;
      const float below = c == 0 ? (e ? ph.x : below_x0) : (c == 1 ? (e ? below_y.y : below_y.x)
                                                                    : (e ? below_z.y : below_z.x));
      const float gp = (phe - below) * float(g.oh[c]);
      out[e] = comp_add(e ? vv[c].y : vv[c].x, e ? lv[c].y : lv[c].x, -(gp * dt), lo + e);
    }
    if (in[c][0] && in[c][1]) {
      *reinterpret_cast<float2 *>(vel[c] + q) = make_float2(out[0], out[1]);
      __nv_bfloat162 l2;
      l2.x = lo[0];
      l2.y = lo[1];
      *reinterpret_cast<__nv_bfloat162 *>(res.c[c] + q) = l2;
    } else if (in[c][0]) {
      vel[c][q] = out[0];
      res.c[c][q] = lo[0];
    } else {
      vel[c][q + 1] = out[1];
      res.c[c][q + 1] = lo[1];
    }
  }
}

// ---- layout conversion and initial fields ----

// lo (float path, compensated state): the residual array of the field, or null.
template <typename T>
__global__ void scatter_kernel(Geometry g, T *dst, const double *src, int ex, int ey, int ez, __nv_bfloat16 *lo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= ex || j >= ey) return;
  const long q = g.idx(i, j, k);
  const double v = src[i + (long)ex * (j + (long)ey * k)];
  if constexpr (std::is_same<T, float>::value) {
    if (lo) {
      dst[q] = comp_split(v, lo + q);
      return;
    }
  }
  dst[q] = T(v);
}

template <typename T>
__global__ void gather_kernel(Geometry g, double *dst, const T *src, int ex, int ey, int ez,
                              const __nv_bfloat16 *lo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= ex || j >= ey) return;
  const long q = g.idx(i, j, k);
  double v = double(src[q]);
  if (lo) v += (double)__bfloat162float(lo[q]);
  dst[i + (long)ex * (j + (long)ey * k)] = v;
}

template <typename T>
__global__ void set_exact_kernel(Geometry g, T *f, int comp, int kind, double t, int ex, int ey, __nv_bfloat16 *lo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= ex || j >= ey) return;
  const long pt[3] = {i, j, k};
  double x[3];
  stag_point(g, comp, pt, x);  // comp 3 (pressure): every axis at nodes
  const long q = g.idx(i, j, k);
  const double v = analytic_value<double>(kind, comp, t, x[0], x[1], x[2], g.Re);
  if constexpr (std::is_same<T, float>::value) {
    if (lo) {
      f[q] = comp_split(v, lo + q);
      return;
    }
  }
  f[q] = T(v);
}

// ---- double-precision reductions ----

__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
  // Non-negative IEEE doubles order like their bit patterns.
  atomicMax(reinterpret_cast<unsigned long long *>(addr), __double_as_longlong(v));
}

template <int NT>
__device__ void block_reduce3(double a, double b, double m, double *acc) {
  __shared__ double sa[NT / 32], sb[NT / 32], sm[NT / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sa[wid] = a, sb[wid] = b, sm[wid] = m;
  __syncthreads();
  if (wid == 0) {
    a = lane < NT / 32 ? sa[lane] : 0.0;
    b = lane < NT / 32 ? sb[lane] : 0.0;
    m = lane < NT / 32 ? sm[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    }
    if (lane == 0) {
      atomicAdd(acc + 0, a);
      atomicAdd(acc + 1, b);
      atomic_max_nonneg(acc + 2, m);
    }
  }
}

// src/Norms.cpp:11-47: velocity interpolated to interior nodes vs the family.
template <typename T>
__global__ void __launch_bounds__(256) velocity_error_kernel(Geometry g, const T *u, const T *v, const T *w, int kind,
                                                             int fn, double t, double *acc, Residual res) {
  const long ni = g.E[0] - 2, nj = g.E[1] - 2, nk = g.E[2] - 2;
  const long n = ni * nj * nk;
  double a = 0, b = 0, m = 0;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (long)gridDim.x * blockDim.x) {
    const long i = 1 + id % ni, j = 1 + (id / ni) % nj, k = 1 + id / (ni * nj);
    const long q = g.idx(i, j, k);
    const double x = g.origin[0] + (double)(g.base[0] + i) * g.h[0];
    const double y = g.origin[1] + (double)(g.base[1] + j) * g.h[1];
    const double z = g.origin[2] + (double)(g.base[2] + k) * g.h[2];
    // the compensated state's value is hi + residual
    auto val = [&](const T *f, int c, long qq) {
      return res.on() ? (double)f[qq] + (double)__bfloat162float(res.c[c][qq]) : (double)f[qq];
    };
    const double iu = (val(u, 0, q) + val(u, 0, q + 1)) / 2.0;
    const double iv = (val(v, 1, q) + val(v, 1, q + g.sy())) / 2.0;
    const double iw = (val(w, 2, q) + val(w, 2, q + g.sz())) / 2.0;
    const double eu = analytic_vector<double>(fn, kind, 0, t, x, y, z, g.Re) - iu;
    const double ev = analytic_vector<double>(fn, kind, 1, t, x, y, z, g.Re) - iv;
    const double ew = analytic_vector<double>(fn, kind, 2, t, x, y, z, g.Re) - iw;
    a += sqrt(eu * eu + ev * ev + ew * ew);
    b += eu * eu + ev * ev + ew * ew;
    m = fmax(m, fmax(fmax(fabs(eu), fabs(ev)), fabs(ew)));
  }
  block_reduce3<256>(a, b, m, acc);
}

// src/Norms.cpp:78-92: pressure on owner points vs the family.
template <typename T>
__global__ void __launch_bounds__(256) pressure_error_kernel(Geometry g, const T *p, int kind, double t, double *acc) {
  const long ni = g.np[0], nj = g.np[1], nk = g.np[2];
  const long n = ni * nj * nk;
  double a = 0, b = 0, m = 0;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (long)gridDim.x * blockDim.x) {
    const long i = g.own_lo[0] + id % ni, j = g.own_lo[1] + (id / ni) % nj, k = g.own_lo[2] + id / (ni * nj);
    const double x = g.origin[0] + (double)(g.base[0] + i) * g.h[0];
    const double y = g.origin[1] + (double)(g.base[1] + j) * g.h[1];
    const double z = g.origin[2] + (double)(g.base[2] + k) * g.h[2];
    const double e = analytic_value<double>(kind, 3, t, x, y, z, g.Re) - (double)p[g.idx(i, j, k)];
    a += fabs(e);
    b += e * e;
    m = fmax(m, fabs(e));
  }
  block_reduce3<256>(a, b, m, acc);
}

// src/PressureEquation.cpp:294-297: sum of (exact - p) over owner points.
template <typename T>
__global__ void __launch_bounds__(256) pressure_diff_kernel(Geometry g, const T *p, int kind, double t, double *acc) {
  const long ni = g.np[0], nj = g.np[1], nk = g.np[2];
  const long n = ni * nj * nk;
  double a = 0;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (long)gridDim.x * blockDim.x) {
    const long i = g.own_lo[0] + id % ni, j = g.own_lo[1] + (id / ni) % nj, k = g.own_lo[2] + id / (ni * nj);
    a += analytic_value<double>(kind, 3, t, g.node(0, i), g.node(1, j), g.node(2, k), g.Re) - (double)p[g.idx(i, j, k)];
  }
  block_reduce3<256>(a, 0.0, 0.0, acc);
}

// src/PressureEquation.cpp:335-342: p += mean difference, every point.
template <typename T>
__global__ void add_shift_kernel(Geometry g, T *p, const double *acc, double count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.E[0] || j >= g.E[1]) return;
  const double shift = acc[0] / count;
  const long q = g.idx(i, j, k);
  p[q] = T((double)p[q] + shift);
}

template <typename T>
__global__ void pressure_gradient_kernel(Geometry g, T *u, T *v, T *w, const T *p) {
  const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = 1 + blockIdx.z;
  T *vel[3] = {u, v, w};
  const long sc[3] = {1, g.sy(), g.sz()};
  const long q = g.idx(i, j, k);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (i >= g.ext(c, 0) - 1 || j >= g.ext(c, 1) - 1 || k >= g.ext(c, 2) - 1) continue;
    vel[c][q] = (p[q] - p[q - sc[c]]) * T(g.oh[c]);
  }
}

inline unsigned cdiv(long a, long b) { return (unsigned)((a + b - 1) / b); }

template <typename T>
Coeffs<T> make_coeffs(const Geometry &g) {
  Coeffs<T> c;
  for (int d = 0; d < 3; ++d) {
    c.o2h[d] = T(g.o2h[d]);
    c.o8h[d] = T(g.o8h[d]);
    c.oh2Re[d] = T(g.oh2Re[d]);
    c.oh[d] = T(g.oh[d]);
  }
  return c;
}

// One stage launch; the compensated variant exists for the float projection stages only.
template <typename T>
struct StageLaunch {
  dim3 grid, blk;
  cudaStream_t s;
  Geometry g;
  Coeffs<T> co;
  Fields<T> F;
  StageCoef<T> K;
  int forcing;
  ForcingEval<T> fe;
  TimeRef tr;
  int sin_slot, kc;
  Residual res;
  const StageProj *proj;
  int *kerr;
  // The tensor maps of the ring fields: the input set's u, v, w and p (the
  // projecting stages' p_in), and phi for the projecting stages.
  // Box widths: kHX (phi kPhiX) for the one-point-per-thread kernels, kQHX
  // for both in the pair kernel.
  bool maps_for(int in_set, bool with_phi, StageMaps &m, bool pair = false) const {
    const T *src[4] = {F.vel(in_set, 0), F.vel(in_set, 1), F.vel(in_set, 2), F.f[kP]};
    if (proj) src[3] = reinterpret_cast<const T *>(proj->p_in);
    const int bx = pair ? kQHX : kHX, pbx = pair ? kQHX : kPhiX;
    for (int f = 0; f < 4; ++f)
      if (!make_field_map(&m.m[f], src[f], (int)sizeof(T), g.PX, g.PY, g.PZ, bx, kHY)) return false;
    m.m[4] = m.m[3];
    return !with_phi || make_field_map(&m.m[4], proj->phi, (int)sizeof(float), g.PX, g.PY, g.PZ, pbx, kPhiRows);
  }
  template <int ST>
  bool go(bool comp) const {
    constexpr int in_set = (ST == kStageY2 || ST == kVelY2 || ST == kVelUStar) ? 0
                           : (ST == kStageY3 || ST == kVelY3)                  ? 1
                                                                               : 2;
    StageMaps m;
    if constexpr (std::is_same<T, float>::value && ST <= kStageUStar) {
      if (comp && proj && !forcing) {
        // two points per thread: 64-point tiles in x
        if (!maps_for(in_set, true, m, true)) return false;
        const int ni = g.Es[0] > g.E[0] ? g.Es[0] : g.E[0];
        const dim3 pgrid(cdiv(ni - 2, kQX), grid.y, grid.z);
        stage_pair_kernel<ST><<<pgrid, blk, 0, s>>>(g, co, F, K, tr, kc, res, *proj, m, kerr);
        return true;
      }
      if (comp && proj) {
        if (!maps_for(in_set, true, m)) return false;
        if (forcing)
          stage_proj_kernel<ST, true><<<grid, blk, 0, s>>>(g, co, F, K, fe, tr, sin_slot, kc, res, *proj, m, kerr);
        else
          stage_proj_kernel<ST, false><<<grid, blk, 0, s>>>(g, co, F, K, fe, tr, sin_slot, kc, res, *proj, m, kerr);
        return true;
      }
    }
    if (!maps_for(in_set, false, m)) return false;
    if constexpr (std::is_same<T, float>::value && ST <= kStageUStar) {
      if (comp) {
        stage_kernel_tiled<T, ST, true><<<grid, blk, 0, s>>>(g, co, F, K, forcing, fe, tr, sin_slot, kc, res, m, kerr);
        return true;
      }
    }
    stage_kernel_tiled<T, ST, false><<<grid, blk, 0, s>>>(g, co, F, K, forcing, fe, tr, sin_slot, kc, res, m, kerr);
    return true;
  }
};

}  // namespace

// ---- launchers ----

template <typename T>
bool launch_stage(const Geometry &g, const Fields<T> &F, StageKind st, const StageScalars<T> &sc,
                  const ForcingTables<T> &ft, int field_kind, TimeRef tr, cudaStream_t s, long long *launches,
                  const Residual &res, const StageProj *proj, int *kerr) {
  const int ni = g.Es[0] > g.E[0] ? g.Es[0] : g.E[0];  // widest extent per axis
  const int nk = g.Es[2] - 2;
  // Planes per CTA: 32, halved (down to 4) while the grid would not fill the
  // GPU's resident slots (twelve CTAs per SM) once, so small grids still
  // occupy every SM; every halving adds a plane of halo reads per CTA.
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
  }
  const long tiles = (long)cdiv(ni - 2, kTX) * cdiv(g.Es[1] - 2, kTY);
  int kc = 32;
  while (kc > 4 && tiles * cdiv(nk, kc) < 12L * sms) kc /= 2;
  const dim3 tgrid(cdiv(ni - 2, kTX), cdiv(g.Es[1] - 2, kTY), cdiv(nk, kc));
  const double dt = sc.dt;
  StageCoef<T> K{};
  switch (st) {
    case kStageY2: {
      const double a1 = 64.0 / 120.0 * dt;
      K = {T(a1), T(0), T(a1), T(0)};
      break;
    }
    case kStageY3: {
      const double a1 = -34.0 / 120.0 * dt, a2 = 50.0 / 120.0 * dt;
      K = {T(a1), T(a2), T(a1 + a2), T(0)};
      break;
    }
    case kStageUStar: {
      const double a2 = -50.0 / 120.0 * dt, a3 = 90.0 / 120.0 * dt;
      K = {T(0), T(a3), T(a2 + a3), T(0)};
      break;
    }
    case kVelY2: {
      const double a21 = (8.0 / 15.0);
      K = {T(dt * a21), T(0), T(0), T(0)};
      break;
    }
    case kVelY3: {
      K = {T(dt), T(1.0 / 4.0), T(1.0 / 4.0), T(5.0 / 12.0)};
      break;
    }
    default: {
      K = {T(dt), T(3.0 / 4.0), T(0), T(0)};
      break;
    }
  }
  ForcingEval<T> fe{};
  fe.tab = ft.tab;
  fe.maxE = ft.maxE;
  fe.st = T(0);
  fe.ct = T(0);
  fe.invRe = T(1.0 / g.Re);
  fe.with_p = sc.forcing == 2;
  fe.tg = sc.forcing == 3;
  fe.alpha = T(sc.alpha);
  const int forcing = ft.tab != nullptr && ((sc.forcing == 1 || sc.forcing == 2) ? field_kind == kFieldSincos
                                                                                  : sc.forcing == 3);
  const Coeffs<T> co = make_coeffs<T>(g);
  const dim3 blk(kTX * kTY);
  const bool comp = res.on() && st <= kStageUStar;
  const StageLaunch<T> L{tgrid, blk, s, g, co, F, K, forcing, fe, tr, sc.sin_slot, kc, res, comp ? proj : nullptr,
                         kerr};
  bool ok = false;
  switch (st) {
    case kStageY2: ok = L.template go<kStageY2>(comp); break;
    case kStageY3: ok = L.template go<kStageY3>(comp); break;
    case kStageUStar: ok = L.template go<kStageUStar>(comp); break;
    case kVelY2: ok = L.template go<kVelY2>(false); break;
    case kVelY3: ok = L.template go<kVelY3>(false); break;
    default: ok = L.template go<kVelUStar>(false); break;
  }
  if (ok && launches) ++*launches;
  return ok;
}

template <typename T>
void launch_apply_bc(const Geometry &g, T *const comp[3], int field_kind, int fn, TimeRef tr, int t_slot,
                     const FaceTables &ft, cudaStream_t s, long long *launches, const Residual &res) {
  const dim3 blk(32, 8, 1);
  int mx = 0;
  for (int d = 0; d < 3; ++d) mx = mx > g.Es[d] ? mx : g.Es[d];
  if (!(g.periodic[0] && g.periodic[1] && g.periodic[2])) {
    const dim3 grid(cdiv(mx, 32), cdiv(mx, 8), 3);
    if (ft.tab)
      bc_faces_kernel<T, true><<<grid, blk, 0, s>>>(g, comp[0], comp[1], comp[2], field_kind, fn, tr, t_slot, ft, res);
    else
      bc_faces_kernel<T, false><<<grid, blk, 0, s>>>(g, comp[0], comp[1], comp[2], field_kind, fn, tr, t_slot, ft,
                                                     res);
    if (launches) ++*launches;
  }
  if (g.periodic[0] || g.periodic[1] || g.periodic[2]) {
    const dim3 grid(cdiv(mx, 32), cdiv(mx, 8), 18);
    periodic_kernel<T><<<grid, blk, 0, s>>>(g, comp[0], comp[1], comp[2], 0, res);
    if (launches) ++*launches;
  }
}

// Precision-independent pieces: compiled in one translation unit only.
#ifdef MIFGPU_STENCIL_SHARED
__global__ void face_table_kernel(Geometry g, int kind, int fn, double tu, double *tab, FaceTables ft) {
  const int c = blockIdx.z / 3, d = blockIdx.z % 3;
  if (g.periodic[d]) return;
  const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
  const long pa = blockIdx.x * blockDim.x + threadIdx.x;
  const long pb = blockIdx.y * blockDim.y + threadIdx.y;
  if (pa >= g.ext(c, a) || pb >= g.ext(c, b)) return;
  for (int s = 0; s < 2; ++s) {
    long pt[3];
    pt[a] = pa;
    pt[b] = pb;
    pt[d] = s == 0 ? 0 : g.ext(c, d) - 1;
    tab[ft.off[fn][c][d][s] + pa + (long)g.ext(c, a) * pb] = face_value<double>(g, c, d, s, pt, kind, fn, tu);
  }
}

void launch_face_tables(const Geometry &g, int field_kind, int fn, double *tab, const FaceTables &ft,
                        cudaStream_t s) {
  int mx = 0;
  for (int d = 0; d < 3; ++d) mx = mx > g.Es[d] ? mx : g.Es[d];
  face_table_kernel<<<dim3(cdiv(mx, 32), cdiv(mx, 8), 9), dim3(32, 8, 1), 0, s>>>(g, field_kind, fn,
                                                                                   family_unit_time(field_kind), tab,
                                                                                   ft);
}

// SINCOS: sin t for both families; ETHIER: exp(-d^2 t / Re) for the velocity
// and its square for the pressure gradient (generators/manufsol.py:35-72).
double family_time_factor(int field_kind, int fn, double t, double Re) {
  if (field_kind == kFieldSincos) return std::sin(t);
  if (field_kind == kFieldEthier) {
    const double d = 1.57079632679489661923;
    return std::exp(-(fn == 0 ? 1.0 : 2.0) * d * d * t / Re);
  }
  return 0.0;
}
double family_unit_time(int field_kind) { return field_kind == kFieldSincos ? 1.57079632679489661923 : 0.0; }
#endif  // MIFGPU_STENCIL_SHARED

template <typename T>
void launch_periodic_scalar(const Geometry &g, T *f, cudaStream_t s, long long *launches) {
  const dim3 blk(32, 8, 1);
  int mx = 0;
  for (int d = 0; d < 3; ++d) mx = mx > g.E[d] ? mx : g.E[d];
  if (g.periodic[0] || g.periodic[1] || g.periodic[2]) {
    const dim3 grid(cdiv(mx, 32), cdiv(mx, 8), 6);
    periodic_kernel<T><<<grid, blk, 0, s>>>(g, f, nullptr, nullptr, 1, Residual{});
    if (launches) ++*launches;
  }
}

template <typename T>
void launch_divergence(const Geometry &g, T *phi, T *const vel[3], double dt, cudaStream_t s, long long *launches,
                       const Residual &res) {
  const dim3 blk(32, 4, 1);
  if constexpr (std::is_same<T, float>::value) {
    if (res.on()) {
      // x pairs from x = 0 up to the owner range's end
      const int pairs = (g.own_lo[0] + g.np[0] + 1) / 2;
      const dim3 grid(cdiv(pairs, 32), cdiv(g.np[1], 4), cdiv(g.np[2], kDivKZComp));
      divergence_pair_kernel<kDivKZComp><<<grid, blk, 0, s>>>(g, phi, vel[0], vel[1], vel[2], T(1.0 / dt), res);
      if (launches) ++*launches;
      return;
    }
  }
  const dim3 grid(cdiv(g.np[0], 32), cdiv(g.np[1], 4), cdiv(g.np[2], kDivKZ));
  divergence_kernel<T><<<grid, blk, 0, s>>>(g, phi, vel[0], vel[1], vel[2], T(1.0 / dt));
  if (launches) ++*launches;
}

template <typename T>
void launch_neumann_flux(const Geometry &g, T *phi, int field_kind, TimeRef tr, int slot_new, int slot_old,
                         cudaStream_t s, long long *launches) {
  const long n = (long)g.E[0] * g.E[1] * g.E[2];
  neumann_flux_serial_kernel<T><<<cdiv(n, 256), 256, 0, s>>>(g, phi, field_kind, tr, slot_new, slot_old);
  if (launches) ++*launches;
}

template <typename T>
void launch_neumann_flux_data(const Geometry &g, T *phi, const GradFaces &gf, int slot, cudaStream_t s,
                              long long *launches) {
  int mx = 0;
  for (int d = 0; d < 3; ++d) mx = mx > g.E[d] ? mx : g.E[d];
  const dim3 blk(32, 8, 1), grid(cdiv(mx, 32), cdiv(mx, 8), 6);
  neumann_flux_data_kernel<T><<<grid, blk, 0, s>>>(g, phi, gf.tab + (long)slot * gf.slot_stride, gf);
  if (launches) ++*launches;
}

template <typename T>
void launch_project(const Geometry &g, T *p, const T *phi, T *const vel[3], double dt, TimeRef tr, unsigned tag,
                    cudaStream_t s, long long *launches, const Residual &res, int *nonfinite) {
  const dim3 blk(32, 4, 1);
  const int ni = g.Es[0] > g.E[0] ? g.Es[0] : g.E[0];
  const dim3 grid(cdiv(ni, 32), cdiv(g.Es[1], 4), cdiv(g.Es[2], kProjKZ));
  if constexpr (std::is_same<T, float>::value) {
    if (res.on()) {
      const dim3 pgrid(cdiv((ni + 1) / 2, 32), cdiv(g.Es[1], 4), (unsigned)g.Es[2]);
      project_pair_kernel<<<pgrid, blk, 0, s>>>(g, p, phi, vel[0], vel[1], vel[2], T(dt), tr, tag, res, nonfinite);
      if (launches) ++*launches;
      return;
    }
  }
  project_kernel<T><<<grid, blk, 0, s>>>(g, p, phi, vel[0], vel[1], vel[2], T(dt), tr, tag, nonfinite);
  if (launches) ++*launches;
}

template <typename T>
void launch_scatter(const Geometry &g, T *dst, const double *src, int ex, int ey, int ez, cudaStream_t s,
                    long long *launches, __nv_bfloat16 *lo) {
  const dim3 blk(32, 8, 1), grid(cdiv(ex, 32), cdiv(ey, 8), (unsigned)ez);
  scatter_kernel<T><<<grid, blk, 0, s>>>(g, dst, src, ex, ey, ez, lo);
  if (launches) ++*launches;
}

template <typename T>
void launch_gather(const Geometry &g, double *dst, const T *src, int ex, int ey, int ez, cudaStream_t s,
                   long long *launches, const __nv_bfloat16 *lo) {
  const dim3 blk(32, 8, 1), grid(cdiv(ex, 32), cdiv(ey, 8), (unsigned)ez);
  gather_kernel<T><<<grid, blk, 0, s>>>(g, dst, src, ex, ey, ez, lo);
  if (launches) ++*launches;
}

template <typename T>
void launch_set_exact(const Geometry &g, T *f, int comp, int field_kind, double t, cudaStream_t s,
                      long long *launches, __nv_bfloat16 *lo) {
  const int ex = comp < 3 ? g.ext(comp, 0) : g.E[0];
  const int ey = comp < 3 ? g.ext(comp, 1) : g.E[1];
  const int ez = comp < 3 ? g.ext(comp, 2) : g.E[2];
  const dim3 blk(32, 8, 1), grid(cdiv(ex, 32), cdiv(ey, 8), (unsigned)ez);
  set_exact_kernel<T><<<grid, blk, 0, s>>>(g, f, comp, field_kind, t, ex, ey, lo);
  if (launches) ++*launches;
}

template <typename T>
void launch_pressure_mean_diff(const Geometry &g, const T *p, int field_kind, double t, double *acc, cudaStream_t s,
                               long long *launches) {
  pressure_diff_kernel<T><<<1024, 256, 0, s>>>(g, p, field_kind, t, acc);
  if (launches) ++*launches;
}

template <typename T>
void launch_add_scalar(const Geometry &g, T *p, const double *shift, cudaStream_t s, long long *launches) {
  const dim3 blk(32, 8, 1), grid(cdiv(g.E[0], 32), cdiv(g.E[1], 8), (unsigned)g.E[2]);
  const double count = (double)((size_t)g.np[0] * (size_t)g.np[1] * (size_t)g.np[2]);
  add_shift_kernel<T><<<grid, blk, 0, s>>>(g, p, shift, count);
  if (launches) ++*launches;
}

template <typename T>
void launch_velocity_errors(const Geometry &g, T *const vel[3], int field_kind, int fn, double t, double *acc,
                            cudaStream_t s, long long *launches, const Residual &res) {
  velocity_error_kernel<T><<<1024, 256, 0, s>>>(g, vel[0], vel[1], vel[2], field_kind, fn, t, acc, res);
  if (launches) ++*launches;
}

template <typename T>
void launch_pressure_errors(const Geometry &g, const T *p, int field_kind, double t, double *acc, cudaStream_t s,
                            long long *launches) {
  pressure_error_kernel<T><<<1024, 256, 0, s>>>(g, p, field_kind, t, acc);
  if (launches) ++*launches;
}

template <typename T>
void launch_pressure_gradient(const Geometry &g, T *const vel[3], const T *p, cudaStream_t s, long long *launches) {
  const dim3 blk(32, 4, 1);
  const int ni = g.Es[0] > g.E[0] ? g.Es[0] : g.E[0];
  const dim3 grid(cdiv(ni - 2, 32), cdiv(g.Es[1] - 2, 4), (unsigned)(g.Es[2] - 2));
  pressure_gradient_kernel<T><<<grid, blk, 0, s>>>(g, vel[0], vel[1], vel[2], p);
  if (launches) ++*launches;
}

#define MIFGPU_INSTANTIATE(T)                                                                                        \
  template bool launch_stage<T>(const Geometry &, const Fields<T> &, StageKind, const StageScalars<T> &,             \
                                const ForcingTables<T> &, int, TimeRef, cudaStream_t, long long *,                   \
                                const Residual &, const StageProj *, int *);                                         \
  template void launch_apply_bc<T>(const Geometry &, T *const[3], int, int, TimeRef, int, const FaceTables &,     \
                                   cudaStream_t, long long *, const Residual &);                                  \
  template void launch_periodic_scalar<T>(const Geometry &, T *, cudaStream_t, long long *);                       \
  template void launch_divergence<T>(const Geometry &, T *, T *const[3], double, cudaStream_t, long long *,       \
                                     const Residual &);                                                            \
  template void launch_neumann_flux<T>(const Geometry &, T *, int, TimeRef, int, int, cudaStream_t, long long *);  \
  template void launch_neumann_flux_data<T>(const Geometry &, T *, const GradFaces &, int, cudaStream_t,            \
                                            long long *);                                                         \
  template void launch_project<T>(const Geometry &, T *, const T *, T *const[3], double, TimeRef, unsigned,      \
                                  cudaStream_t, long long *, const Residual &, int *);                            \
  template void launch_scatter<T>(const Geometry &, T *, const double *, int, int, int, cudaStream_t, long long *,  \
                                  __nv_bfloat16 *);                                                               \
  template void launch_gather<T>(const Geometry &, double *, const T *, int, int, int, cudaStream_t, long long *,  \
                                 const __nv_bfloat16 *);                                                          \
  template void launch_set_exact<T>(const Geometry &, T *, int, int, double, cudaStream_t, long long *,            \
                                    __nv_bfloat16 *);                                                             \
  template void launch_pressure_mean_diff<T>(const Geometry &, const T *, int, double, double *, cudaStream_t,     \
                                             long long *);                                                         \
  template void launch_add_scalar<T>(const Geometry &, T *, const double *, cudaStream_t, long long *);            \
  template void launch_velocity_errors<T>(const Geometry &, T *const[3], int, int, double, double *, cudaStream_t, \
                                          long long *, const Residual &);                                          \
  template void launch_pressure_errors<T>(const Geometry &, const T *, int, double, double *, cudaStream_t,        \
                                          long long *);                                                            \
  template void launch_pressure_gradient<T>(const Geometry &, T *const[3], const T *, cudaStream_t, long long *);

}  // namespace mifgpu
