// Discrete adjoint of the projection step (sm_103a): the transposes of every
// linear map of src/Timestep.cpp:97-141 and of the linearised momentum
// right-hand side of include/MomentumEquation.h:42-255, as gather kernels
// (one thread per output point, no atomics, deterministic).
//
// The reference has no adjoint; this is an extension. Notation:
//   R_c(P)  momentum right-hand side of component c at its interior point P
//   G       one-sided pressure gradient onto interior velocity points
//   D       divergence at the pressure owner points
//   M       the spectral Poisson solve on the owner block
// Adjoint weights of R_c are zero outside the interior of component c; the
// split kernel stores them so, and the gathers rely on it instead of masking
// each read. Reductions (the loss, d loss / d alpha) go through per-block
// partial sums added in a fixed order, so results are bitwise reproducible.
//
// M is not symmetric on a Neumann (DCT-I) axis: the reflection closure of
// the Laplacian there is symmetric only in the trapezoid inner product with
// weight 1/2 at both end points. With W the product of those weights,
// M^T = W M W^-1, so the adjoint solve is the forward solve between a
// division by W (folded into the gradient transpose that builds its
// right-hand side) and a multiplication by W (folded into the divergence
// transpose that reads its solution).
#pragma once

#include <algorithm>

#include "common.cuh"
#include "tma.cuh"

namespace mifgpu {

namespace adj {

__device__ __forceinline__ bool interior(const Geometry &g, int c, int i, int j, int k) {
  return i >= 1 && j >= 1 && k >= 1 && i < g.ext(c, 0) - 1 && j < g.ext(c, 1) - 1 && k < g.ext(c, 2) - 1;
}

__device__ __forceinline__ bool owner(const Geometry &g, int i, int j, int k) {
  return i >= g.own_lo[0] && i < g.own_lo[0] + g.np[0] && j >= g.own_lo[1] && j < g.own_lo[1] + g.np[1] &&
         k >= g.own_lo[2] && k < g.own_lo[2] + g.np[2];
}

// Trapezoid weight of a pressure point: 1/2 per Neumann axis on which it is
// an end point; returned as the number of such axes (the weight is 2^-nb, a
// power of two, so scaling by it or its inverse is exact in any precision).
__device__ __forceinline__ int trap_halvings(const Geometry &g, int i, int j, int k) {
  const int q[3] = {i, j, k};
  int nb = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (!g.periodic[d] && (q[d] == 0 || q[d] == g.E[d] - 1)) ++nb;
  return nb;
}
template <typename T>
__device__ __forceinline__ T trap_weight(const Geometry &g, int i, int j, int k) {
  return T(1) / T(1 << trap_halvings(g, i, j, k));
}

// ---- transposed momentum right-hand side, shared-memory tiled ----
//
// A CTA owns a TX x TY tile of (i, j) and marches through kc planes of k,
// like the forward stage kernel. The three adjoint weights mu_c and the three
// linearisation fields V_c live in a ring of six shared-memory planes per
// field (k-2 .. k+2 and the plane being prefetched), each with a two-point
// halo in x and y: the gather reads V up to two points away along one axis
// (Avg_{d,c} at P = Q + e_d, and the cross terms at P = Q - e_f). mu is zero
// off the interior of its component in memory (the split kernel writes those
// zeros and the padding is cleared once), so no read needs a mask.
// A plane tile is one TMA box of kAHX x kAHY elements from (i0 - kAXO,
// j0 - kAH): four columns before the tile in x, so the box starts 16-byte
// aligned (i0 is a multiple of 32), two rows before it in y; boxes outside
// the field read zeros. A slot is 1920 bytes in float (3840 in double), so
// every slot starts 128-byte aligned.
constexpr int kATX = 32, kATY = 8, kAH = 2, kAXO = 4;
constexpr int kAHX = kATX + 2 * kAXO, kAHY = kATY + 2 * kAH, kAPL = kAHX * kAHY;
constexpr int kASlots = 6;
static_assert((kAPL * 4) % 128 == 0, "128-byte aligned ring slots");

template <typename T>
struct AdjRing {
  T f[6][kASlots][kAPL];  // mu_u, mu_v, mu_w, V_u, V_v, V_w; slot (k mod 6); tile
  uint64_t bar[kASlots];  // one TMA barrier per slot
};

// Tensor maps of mu_u, mu_v, mu_w, V_u, V_v, V_w.
struct AdjMaps {
  CUtensorMap m[6];
};

template <typename T>
struct ATap {
  const AdjRing<T> *r;
  int base;      // (ty + kAH) * kAHX + tx + kAXO
  int slot[5];   // slot of plane k + dk for dk = -2 .. 2
  __device__ __forceinline__ T mu(int c, int di, int dj, int dk) const {
    return r->f[c][slot[dk + 2]][base + dj * kAHX + di];
  }
  __device__ __forceinline__ T v(int c, int di, int dj, int dk) const {
    return r->f[3 + c][slot[dk + 2]][base + dj * kAHX + di];
  }
};

// Avg_{d,c}(P) = V_d(P) + V_d(P+e_d) + V_d(P-e_c) + V_d(P-e_c+e_d) at P = Q + (a, b, e).
template <typename T, int D, int C>
__device__ __forceinline__ T avg_tap(const ATap<T> &A, int a, int b, int e) {
  constexpr int di = D == 0, dj = D == 1, dk = D == 2;
  constexpr int ci = C == 0, cj = C == 1, ck = C == 2;
  return A.v(D, a, b, e) + A.v(D, a + di, b + dj, e + dk) + A.v(D, a - ci, b - cj, e - ck) +
         A.v(D, a - ci + di, b - cj + dj, e - ck + dk);
}

// Cross term of R_C read through Avg_{F,C}: sum over P in {Q, Q-e_F, Q+e_C, Q+e_C-e_F}
// of mu_C(P) (V_C(P+e_F) - V_C(P-e_F)) o8h_F.
template <typename T, int F, int C>
__device__ __forceinline__ T cross_tap(const ATap<T> &A) {
  constexpr int fi = F == 0, fj = F == 1, fk = F == 2;
  constexpr int ci = C == 0, cj = C == 1, ck = C == 2;
  T s = T(0);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int a = (r >= 2 ? ci : 0) - (r & 1 ? fi : 0);
    const int b = (r >= 2 ? cj : 0) - (r & 1 ? fj : 0);
    const int e = (r >= 2 ? ck : 0) - (r & 1 ? fk : 0);
    s += A.mu(C, a, b, e) * (A.v(C, a + fi, b + fj, e + fk) - A.v(C, a - fi, b - fj, e - fk));
  }
  return s;
}

// Self-convection of R_F by V_D (D != F): mu_F(Q-e_D) Avg_{D,F}(Q-e_D) - mu_F(Q+e_D) Avg_{D,F}(Q+e_D).
template <typename T, int F, int D>
__device__ __forceinline__ T conv_tap(const ATap<T> &A) {
  constexpr int di = D == 0, dj = D == 1, dk = D == 2;
  return A.mu(F, -di, -dj, -dk) * avg_tap<T, D, F>(A, -di, -dj, -dk) -
         A.mu(F, di, dj, dk) * avg_tap<T, D, F>(A, di, dj, dk);
}

// (R'(V)^T mu)_F at the tap's point, with
//   R_c(P) = - V_c(P) (V_c(P+e_c) - V_c(P-e_c)) o2h_c
//            - sum_{d != c} Avg_{d,c}(P) (V_c(P+e_d) - V_c(P-e_d)) o8h_d
//            + sum_d (V_c(P+e_d) - 2 V_c(P) + V_c(P-e_d)) oh2Re_d
template <typename T, int F>
__device__ __forceinline__ T rhs_adjoint_tap(const ATap<T> &A, const Coeffs<T> &co) {
  constexpr int fi = F == 0, fj = F == 1, fk = F == 2;
  constexpr int D1 = F == 0 ? 1 : 0, D2 = F == 2 ? 1 : 2;  // the two other axes
  const T m0 = A.mu(F, 0, 0, 0);
  const T mm = A.mu(F, -fi, -fj, -fk), mp = A.mu(F, fi, fj, fk);
  // self-advection along F
  T acc = (mp * A.v(F, fi, fj, fk) - mm * A.v(F, -fi, -fj, -fk) -
           m0 * (A.v(F, fi, fj, fk) - A.v(F, -fi, -fj, -fk))) * co.o2h[F];
  // convection of F by the other two components
  acc -= conv_tap<T, F, D1>(A) * co.o8h[D1];
  acc -= conv_tap<T, F, D2>(A) * co.o8h[D2];
  // diffusion
  acc += (mp - T(2) * m0 + mm) * co.oh2Re[F];
  acc += (A.mu(F, D1 == 0, D1 == 1, D1 == 2) - T(2) * m0 + A.mu(F, -(D1 == 0), -(D1 == 1), -(D1 == 2))) *
         co.oh2Re[D1];
  acc += (A.mu(F, D2 == 0, D2 == 1, D2 == 2) - T(2) * m0 + A.mu(F, -(D2 == 0), -(D2 == 1), -(D2 == 2))) *
         co.oh2Re[D2];
  // the other components' convection reads V_F through their averages
  acc -= (cross_tap<T, F, D1>(A) + cross_tap<T, F, D2>(A)) * co.o8h[F];
  return acc;
}

// lam_c += (R'(V)^T mu)_c on every point of the three fields.
// The ring is filled by TMA: thread 0 loads a plane's six tiles into its slot
// on the slot's mbarrier, and every thread waits on the barrier before
// reading the plane (plane kk is the ((kk - kfirst) / 6)-th load of its
// slot). A wait that gives up sets *kerr and the thread skips its later
// waits, so the CTA still reaches every barrier and ends.
template <typename T>
__global__ void __launch_bounds__(kATX *kATY) rhs_adjoint_tiled(Geometry g, Coeffs<T> co, T *l0, T *l1, T *l2,
                                                                int kc, const __grid_constant__ AdjMaps maps,
                                                                int *kerr) {
  extern __shared__ __align__(16) unsigned char adj_smem[];
  AdjRing<T> &ring =
      *reinterpret_cast<AdjRing<T> *>(adj_smem + ((128 - (smem_u32(adj_smem) & 127)) & 127));
  const int tx = threadIdx.x % kATX, ty = threadIdx.x / kATX;
  const int i0 = blockIdx.x * kATX, j0 = blockIdx.y * kATY;
  const int kbeg = blockIdx.z * kc, kend = min(kbeg + kc, g.Es[2]);
  const int kfirst = kbeg - 2;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int b = 0; b < kASlots; ++b) mbar_init(&ring.bar[b], 1);
    mbar_init_fence();
  }
  __syncthreads();
  auto slot_of = [](int kk) { return (kk + 2 * kASlots) % kASlots; };
  auto load_plane = [&](int kk) {  // thread 0
    const int sl = slot_of(kk);
    mbar_expect_tx(&ring.bar[sl], (unsigned)(6 * kAPL * sizeof(T)));
#pragma unroll
    for (int f = 0; f < 6; ++f) tma_load_3d(&ring.f[f][sl][0], &maps.m[f], i0 - kAXO, j0 - kAH, kk, &ring.bar[sl]);
  };
  bool tma_ok = true;
  auto wait_plane = [&](int kk) {
    if (tma_ok && !mbar_wait(&ring.bar[slot_of(kk)], ((kk - kfirst) / kASlots) & 1)) {
      tma_ok = false;
      if (kerr) atomicExch(kerr, 1);
    }
  };
  if (threadIdx.x == 0)
    for (int kk = kbeg - 2; kk <= kbeg + 2; ++kk) load_plane(kk);
  for (int kk = kbeg - 2; kk <= kbeg + 1; ++kk) wait_plane(kk);
  const int i = i0 + tx, j = j0 + ty;
  T *lam[3] = {l0, l1, l2};
  ATap<T> A;
  A.r = &ring;
  A.base = (ty + kAH) * kAHX + tx + kAXO;
  for (int k = kbeg; k < kend; ++k) {
    // plane k + 3 (needed while k + 3 <= kend + 1) into the slot of plane
    // k - 3, which the barrier that ended the previous iteration released
    if (threadIdx.x == 0 && k + 3 <= kend + 1) {
      fence_async_shared();
      load_plane(k + 3);
    }
    wait_plane(k + 2);
#pragma unroll
    for (int dk = -2; dk <= 2; ++dk) A.slot[dk + 2] = (k + dk + 2 * kASlots) % kASlots;
    const long q = g.idx(i, j, k);
    if (i < g.ext(0, 0) && j < g.ext(0, 1) && k < g.ext(0, 2)) lam[0][q] += rhs_adjoint_tap<T, 0>(A, co);
    if (i < g.ext(1, 0) && j < g.ext(1, 1) && k < g.ext(1, 2)) lam[1][q] += rhs_adjoint_tap<T, 1>(A, co);
    if (i < g.ext(2, 0) && j < g.ext(2, 1) && k < g.ext(2, 2)) lam[2][q] += rhs_adjoint_tap<T, 2>(A, co);
    __syncthreads();  // the next iteration refills the slot of plane k - 2
  }
}

// out(r) = (add(r) + scale (G^T mu)(r)) / (weighted ? W(r) : 1) on the pressure
// extents, (G^T mu)(r) = sum_c oh_c (mu_c(r) [r interior of c] - mu_c(r+e_c) [r+e_c interior of c]).
// out may alias add.
template <typename T>
__global__ void grad_adjoint_kernel(Geometry g, T *out, const T *add, const T *m0, const T *m1, const T *m2,
                                    T scale, int weighted) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.E[0] || j >= g.E[1]) return;
  const T *mu[3] = {m0, m1, m2};
  const long q = g.idx(i, j, k);
  const long st[3] = {1, g.sy(), g.sz()};
  T acc = T(0);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    T a = interior(g, c, i, j, k) ? mu[c][q] : T(0);
    if (interior(g, c, i + (c == 0), j + (c == 1), k + (c == 2))) a -= mu[c][q + st[c]];
    acc += a * T(g.oh[c]);
  }
  T v = scale * acc;
  if (add) v += add[q];
  if (weighted) v *= T(1 << trap_halvings(g, i, j, k));
  out[q] = v;
}

// out_c(q) = in_c(q) + scale (D^T (W rho))_c(q), (D^T r)_c(q) = oh_c (r(q-e_c) - r(q)),
// r taken as zero off the owner block. out may alias in.
template <typename T>
__global__ void div_adjoint_kernel(Geometry g, T *o0, T *o1, T *o2, const T *i0, const T *i1, const T *i2,
                                   const T *rho, T scale) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  T *out[3] = {o0, o1, o2};
  const T *in[3] = {i0, i1, i2};
  const long q = g.idx(i, j, k);
  const long st[3] = {1, g.sy(), g.sz()};
  const T r0 = owner(g, i, j, k) ? rho[q] * trap_weight<T>(g, i, j, k) : T(0);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (i >= g.ext(c, 0) || j >= g.ext(c, 1) || k >= g.ext(c, 2)) continue;
    const int im = i - (c == 0), jm = j - (c == 1), km = k - (c == 2);
    const T rm = owner(g, im, jm, km) ? rho[q - st[c]] * trap_weight<T>(g, im, jm, km) : T(0);
    out[c][q] = in[c][q] + scale * (rm - r0) * T(g.oh[c]);
  }
}

// Adjoint of the periodic copies of all axes (src/StaggeredTensor.cpp:221-257).
// Forward, along x, then y, then z: a[0] = a[E-2], a[E-1] = a[1]. The adjoint
// runs z, y, x, and along one axis does lam[1] += lam[E-1],
// lam[E-2] += lam[0], then clears both ghosts. Done at once as a gather:
// every ghost value ends on one non-ghost point Q (its image along every
// periodic axis where it is a ghost). The thread of Q sums the 2^n sources in
// the sequential association,
//   V_z(p) = lam(p) + lam(p, z ghost),  V_zy(p) = V_z(p) + V_z(p, y ghost),
//   lam(Q) = V_zy(Q) + V_zy(Q, x ghost),
// so the result is bitwise the one of the three passes, and then clears the
// ghosts it read; no other thread reads them. blockIdx.z = comp * 6 + face:
// Q on the face plane 1 / E-2 of periodic axis d, counted only on its first
// such axis.
template <typename T>
__global__ void periodic_fold_adjoint_kernel(Geometry g, T *f0, T *f1, T *f2, int scalar) {
  const int c = blockIdx.z / 6, face = blockIdx.z % 6, d = face / 2, side = face % 2;
  T *f = c == 0 ? f0 : (c == 1 ? f1 : f2);
  if (!f || !g.periodic[d]) return;
  int ex[3];
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) ex[ax] = scalar ? g.E[ax] : g.ext(c, ax);
  const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
  // the other two axes: non-ghost points of a periodic axis, all of another
  const int la = g.periodic[a] ? 1 : 0, lb = g.periodic[b] ? 1 : 0;
  const int na = g.periodic[a] ? ex[a] - 2 : ex[a], nb = g.periodic[b] ? ex[b] - 2 : ex[b];
  const int pa = blockIdx.x * blockDim.x + threadIdx.x, pb = blockIdx.y * blockDim.y + threadIdx.y;
  if (pa >= na || pb >= nb) return;
  int q[3];
  q[d] = side == 0 ? 1 : ex[d] - 2;
  q[a] = la + pa;
  q[b] = lb + pb;
  bool has[3];
  int gh[3];
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    has[ax] = g.periodic[ax] && (q[ax] == 1 || q[ax] == ex[ax] - 2);
    gh[ax] = q[ax] == 1 ? ex[ax] - 1 : 0;
  }
  for (int ax = 0; ax < d; ++ax)
    if (has[ax]) return;  // Q belongs to an earlier axis's face
  // sources: bit ax of s set = coordinate ax replaced by its ghost
  auto at = [&](int s) -> long {
    const int x = (s & 1) ? gh[0] : q[0], y = (s & 2) ? gh[1] : q[1], z = (s & 4) ? gh[2] : q[2];
    return g.idx(x, y, z);
  };
  auto vz = [&](int s) { return has[2] ? f[at(s)] + f[at(s | 4)] : f[at(s)]; };
  auto vzy = [&](int s) { return has[1] ? vz(s) + vz(s | 2) : vz(s); };
  const T v = has[0] ? vzy(0) + vzy(1) : vzy(0);
  f[at(0)] = v;
  for (int s = 1; s < 8; ++s) {
    if (((s & 1) && !has[0]) || ((s & 2) && !has[1]) || ((s & 4) && !has[2])) continue;
    f[at(s)] = T(0);
  }
}

// Adjoint of the Dirichlet faces: those points were overwritten with data.
template <typename T>
__global__ void dirichlet_adjoint_kernel(Geometry g, T *f0, T *f1, T *f2) {
  const long i = blockIdx.x * blockDim.x + threadIdx.x;
  const long j = blockIdx.y * blockDim.y + threadIdx.y;
  const long k = blockIdx.z;
  T *f[3] = {f0, f1, f2};
  const long q3[3] = {i, j, k};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (i >= g.ext(c, 0) || j >= g.ext(c, 1) || k >= g.ext(c, 2)) continue;
    bool face = false;
    for (int d = 0; d < 3; ++d)
      if (!g.periodic[d] && (q3[d] == 0 || q3[d] == g.ext(c, d) - 1)) face = true;
    if (face) f[c][g.idx(i, j, k)] = T(0);
  }
}

// Sum of v over the block (32 x 8 threads) in a fixed order, written to
// part[linear block index] by thread 0: deterministic partial sums.
template <typename A>
__device__ __forceinline__ void block_partial(A v, double *part) {
  __shared__ double w[8];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  if ((t & 31) == 0) w[t >> 5] = (double)v;
  __syncthreads();
  if (t == 0) {
    double s = 0.0;
    for (int q = 0; q < 8; ++q) s += w[q];
    part[blockIdx.x + (long)gridDim.x * (blockIdx.y + (long)gridDim.y * blockIdx.z)] = s;
  }
}

// *out (+)= sum of part[0 .. n) in a fixed order (one block of 256 threads).
__global__ void sum_partials_kernel(const double *part, long n, double *out, int accumulate) {
  __shared__ double w[256];
  double v = 0.0;
  for (long q = threadIdx.x; q < n; q += 256) v += part[q];
  w[threadIdx.x] = v;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) w[threadIdx.x] += w[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = accumulate ? *out + w[0] : w[0];
}

// Split of the adjoint of one stage's pre-projection set X (lx, zero off the
// interior) on the interior points:
//   mu   = a lx + b pend      (adjoint weights of this stage's R)
//   pend = a2 lx              (when write_pend: the share of an earlier R)
// mu is written as 0 on the other points of each component's extents (the
// tiled gather relies on it). When tab is given, each block writes its share
// of sum mu_c F_c to part[], F the Taylor-Green body-force pattern
// (sin x cos y cos z, -cos x sin y cos z, 0).
template <typename T>
__global__ void split_kernel(Geometry g, T *m0, T *m1, T *m2, T *p0, T *p1, T *p2, const T *x0, const T *x1,
                             const T *x2, T a, T b, T a2, int write_pend, const T *tab, int maxE, double *part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  T *mu[3] = {m0, m1, m2}, *pend[3] = {p0, p1, p2};
  const T *lx[3] = {x0, x1, x2};
  const long q = g.idx(i, j, k);
  T f = T(0);  // this point's share of mu . F (warp sums in T, block sums in double)
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (i >= g.ext(c, 0) || j >= g.ext(c, 1) || k >= g.ext(c, 2)) continue;
    if (!interior(g, c, i, j, k)) {
      mu[c][q] = T(0);
      continue;
    }
    const T x = lx[c][q];
    T m = a * x;
    if (b != T(0)) m += b * pend[c][q];
    mu[c][q] = m;
    if (write_pend) pend[c][q] = a2 * x;
    if (tab && c < 2) {
      auto S = [&](int ax, int face, int n) { return tab[((ax * 2 + face) * 2 + 0) * maxE + n]; };
      auto C = [&](int ax, int face, int n) { return tab[((ax * 2 + face) * 2 + 1) * maxE + n]; };
      if (c == 0)
        f += m * (S(0, 1, i) * C(1, 0, j) * C(2, 0, k));
      else
        f -= m * (C(0, 0, i) * S(1, 1, j) * C(2, 0, k));
    }
  }
  if (tab) block_partial(f, part);
}

// Kinetic energy in an axis-aligned box at the staggered points:
//   L = 1/2 vol sum_c sum_{q interior of c, position in box} u_c(q)^2
// lam_c(q) = vol u_c(q) there and 0 on every other point; each block writes
// its share of L to part[].
template <typename T>
__global__ void ke_seed_kernel(Geometry g, const T *u0, const T *u1, const T *u2, T *l0, T *l1, T *l2, double x0,
                               double x1, double y0, double y1, double z0, double z1, double *part) {
  const long i = blockIdx.x * blockDim.x + threadIdx.x;
  const long j = blockIdx.y * blockDim.y + threadIdx.y;
  const long k = blockIdx.z;
  const T *u[3] = {u0, u1, u2};
  T *l[3] = {l0, l1, l2};
  const double vol = g.h[0] * g.h[1] * g.h[2];
  double a = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (i >= g.ext(c, 0) || j >= g.ext(c, 1) || k >= g.ext(c, 2)) continue;
    const long q = g.idx(i, j, k);
    const double x = c == 0 ? g.face(0, i) : g.node(0, i);
    const double y = c == 1 ? g.face(1, j) : g.node(1, j);
    const double z = c == 2 ? g.face(2, k) : g.node(2, k);
    const bool in = interior(g, c, i, j, k) && x >= x0 && x <= x1 && y >= y0 && y <= y1 && z >= z0 && z <= z1;
    const double v = (double)u[c][q];
    l[c][q] = in ? T(vol * v) : T(0);
    if (in) a += 0.5 * vol * v * v;
  }
  block_partial(a, part);
}

inline unsigned cdiv_u(long a, long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace adj

// Host launchers; every launch adds one to *cnt.
template <typename T>
struct AdjointOps {
  // Blocks of 32 x 8 threads over the widest extent per axis, one z plane per grid z.
  static dim3 box_grid(const Geometry &g) {
    const int nx = std::max(g.Es[0], g.E[0]);
    return dim3(adj::cdiv_u(nx, 32), adj::cdiv_u(g.Es[1], 8), (unsigned)g.Es[2]);
  }
  static Coeffs<T> coeffs(const Geometry &g) {
    Coeffs<T> co;
    for (int d = 0; d < 3; ++d) {
      co.o2h[d] = T(g.o2h[d]);
      co.o8h[d] = T(g.o8h[d]);
      co.oh2Re[d] = T(g.oh2Re[d]);
      co.oh[d] = T(g.oh[d]);
    }
    return co;
  }
  // the ring and 128 bytes to align it
  static constexpr size_t kRingSmem = sizeof(adj::AdjRing<T>) + 128;
  // Kernel attributes; call once before the first launch (outside stream capture).
  static cudaError_t prepare() {
    return cudaFuncSetAttribute(adj::rhs_adjoint_tiled<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kRingSmem);
  }
  // Needs mu zero off each component's interior, padding included, and
  // prepare(). False (nothing launched) if a tensor map was rejected; `kerr`
  // (device, may be null) as for the stage kernels.
  static bool rhs_adjoint(const Geometry &g, T *const lam[3], const T *const mu[3], const T *const V[3],
                          cudaStream_t s, long long *cnt, int *kerr = nullptr) {
    const int nx = std::max(g.Es[0], g.E[0]);
    // 8 planes per CTA below 256 planes: more, shorter CTAs; at 128^3 the
    // reverse step measured 0.734 / 0.762 / 0.777 ms for 8 / 16 / 32 (FP32).
    const int kc = g.Es[2] >= 256 ? 32 : 8;
    const dim3 grid(adj::cdiv_u(nx, adj::kATX), adj::cdiv_u(g.Es[1], adj::kATY), adj::cdiv_u(g.Es[2], kc));
    adj::AdjMaps maps;
    const T *src[6] = {mu[0], mu[1], mu[2], V[0], V[1], V[2]};
    for (int f = 0; f < 6; ++f)
      if (!make_field_map(&maps.m[f], src[f], (int)sizeof(T), g.PX, g.PY, g.PZ, adj::kAHX, adj::kAHY)) return false;
    adj::rhs_adjoint_tiled<T><<<grid, adj::kATX * adj::kATY, kRingSmem, s>>>(g, coeffs(g), lam[0], lam[1], lam[2],
                                                                             kc, maps, kerr);
    ++*cnt;
    return true;
  }
  static void grad_adjoint(const Geometry &g, T *out, const T *add, const T *const mu[3], double scale,
                           bool weighted, cudaStream_t s, long long *cnt) {
    const dim3 grid(adj::cdiv_u(g.E[0], 32), adj::cdiv_u(g.E[1], 8), (unsigned)g.E[2]);
    adj::grad_adjoint_kernel<T><<<grid, dim3(32, 8), 0, s>>>(g, out, add, mu[0], mu[1], mu[2], T(scale),
                                                              weighted ? 1 : 0);
    ++*cnt;
  }
  static void div_adjoint(const Geometry &g, T *const out[3], const T *const in[3], const T *rho, double scale,
                          cudaStream_t s, long long *cnt) {
    adj::div_adjoint_kernel<T><<<box_grid(g), dim3(32, 8), 0, s>>>(g, out[0], out[1], out[2], in[0], in[1], in[2],
                                                                   rho, T(scale));
    ++*cnt;
  }
  // Boundary-fill adjoint: the periodic copies in reverse order (z, y, x),
  // then the Dirichlet faces.
  static void bc_adjoint(const Geometry &g, T *const f[3], cudaStream_t s, long long *cnt) {
    int mx = 0;
    for (int d = 0; d < 3; ++d) mx = std::max(mx, g.Es[d]);
    if (g.periodic[0] || g.periodic[1] || g.periodic[2]) {
      adj::periodic_fold_adjoint_kernel<T><<<dim3(adj::cdiv_u(mx, 32), adj::cdiv_u(mx, 8), 18), dim3(32, 8), 0, s>>>(
          g, f[0], f[1], f[2], 0);
      ++*cnt;
    }
    if (!(g.periodic[0] && g.periodic[1] && g.periodic[2])) {
      adj::dirichlet_adjoint_kernel<T><<<box_grid(g), dim3(32, 8), 0, s>>>(g, f[0], f[1], f[2]);
      ++*cnt;
    }
  }
  static void periodic_scalar_adjoint(const Geometry &g, T *f, cudaStream_t s, long long *cnt) {
    int mx = 0;
    for (int d = 0; d < 3; ++d) mx = std::max(mx, g.E[d]);
    if (g.periodic[0] || g.periodic[1] || g.periodic[2]) {
      adj::periodic_fold_adjoint_kernel<T><<<dim3(adj::cdiv_u(mx, 32), adj::cdiv_u(mx, 8), 6), dim3(32, 8), 0, s>>>(
          g, f, nullptr, nullptr, 1);
      ++*cnt;
    }
  }
  // Blocks of box_grid: the length of the partial-sum array.
  static long box_blocks(const Geometry &g) {
    const dim3 b = box_grid(g);
    return (long)b.x * b.y * b.z;
  }
  // With tab: *acc += sum mu . F, through part[box_blocks] in a fixed order.
  static void split(const Geometry &g, T *const mu[3], T *const pend[3], const T *const lx[3], double a, double b,
                    double a2, bool write_pend, const T *tab, int maxE, double *part, double *acc, cudaStream_t s,
                    long long *cnt) {
    adj::split_kernel<T><<<box_grid(g), dim3(32, 8), 0, s>>>(g, mu[0], mu[1], mu[2], pend[0], pend[1], pend[2],
                                                             lx[0], lx[1], lx[2], T(a), T(b), T(a2),
                                                             write_pend ? 1 : 0, tab, maxE, part);
    ++*cnt;
    if (tab) {
      adj::sum_partials_kernel<<<1, 256, 0, s>>>(part, box_blocks(g), acc, 1);
      ++*cnt;
    }
  }
  // *acc = the loss, through part[box_blocks].
  static void ke_seed(const Geometry &g, const T *const u[3], T *const lam[3], const double box[6], double *part,
                      double *acc, cudaStream_t s, long long *cnt) {
    adj::ke_seed_kernel<T><<<box_grid(g), dim3(32, 8), 0, s>>>(g, u[0], u[1], u[2], lam[0], lam[1], lam[2], box[0],
                                                               box[1], box[2], box[3], box[4], box[5], part);
    adj::sum_partials_kernel<<<1, 256, 0, s>>>(part, box_blocks(g), acc, 0);
    *cnt += 2;
  }
};

}  // namespace mifgpu
