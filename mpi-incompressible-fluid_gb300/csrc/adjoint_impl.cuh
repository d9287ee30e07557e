// Discrete adjoint of the projection step (sm_103a): the transposes of every
// linear map of src/Timestep.cpp:97-141 and of the linearised momentum
// right-hand side of include/MomentumEquation.h:42-255, as gather kernels
// (one thread per output point, no atomics on fields, deterministic).
//
// The reference has no adjoint; this is an extension. Notation:
//   R_c(P)  momentum right-hand side of component c at its interior point P
//   G       one-sided pressure gradient onto interior velocity points
//   D       divergence at the pressure owner points
//   M       the spectral Poisson solve on the owner block
// Adjoint weights of R_c are zero outside the interior of component c, so
// every gather masks its reads with the interior predicate; that also keeps
// every state read inside the field.
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

namespace mifgpu {

namespace adj {

__device__ __forceinline__ bool interior(const Geometry &g, int c, long i, long j, long k) {
  return i >= 1 && j >= 1 && k >= 1 && i < g.ext(c, 0) - 1 && j < g.ext(c, 1) - 1 && k < g.ext(c, 2) - 1;
}

__device__ __forceinline__ bool owner(const Geometry &g, long i, long j, long k) {
  return i >= g.own_lo[0] && i < g.own_lo[0] + g.np[0] && j >= g.own_lo[1] && j < g.own_lo[1] + g.np[1] &&
         k >= g.own_lo[2] && k < g.own_lo[2] + g.np[2];
}

// Trapezoid weight of a pressure point: 1/2 per Neumann axis on which it is
// an end point.
__device__ __forceinline__ double trap_weight(const Geometry &g, long i, long j, long k) {
  const long q[3] = {i, j, k};
  double w = 1.0;
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (!g.periodic[d] && (q[d] == 0 || q[d] == g.E[d] - 1)) w *= 0.5;
  return w;
}

template <typename T>
struct View {
  Geometry g;
  const T *mu[3];  // adjoint weights of R_c
  const T *V[3];   // state R was linearised at
  __device__ __forceinline__ T M(int c, long i, long j, long k) const {
    return interior(g, c, i, j, k) ? mu[c][g.idx(i, j, k)] : T(0);
  }
  __device__ __forceinline__ T S(int c, long i, long j, long k) const { return V[c][g.idx(i, j, k)]; }
};

// Avg_{d,c}(P) = V_d(P) + V_d(P+e_d) + V_d(P-e_c) + V_d(P-e_c+e_d): the four
// V_d values the convection of component c averages (d != c).
template <typename T>
__device__ __forceinline__ T avg_dc(const View<T> &A, int d, int c, long i, long j, long k) {
  const long di = d == 0, dj = d == 1, dk = d == 2;
  const long ci = c == 0, cj = c == 1, ck = c == 2;
  return A.S(d, i, j, k) + A.S(d, i + di, j + dj, k + dk) + A.S(d, i - ci, j - cj, k - ck) +
         A.S(d, i - ci + di, j - cj + dj, k - ck + dk);
}

// (R'(V)^T mu)_f at Q = (i, j, k), with
//   R_c(P) = - V_c(P) (V_c(P+e_c) - V_c(P-e_c)) o2h_c
//            - sum_{d != c} Avg_{d,c}(P) (V_c(P+e_d) - V_c(P-e_d)) o8h_d
//            + sum_d (V_c(P+e_d) - 2 V_c(P) + V_c(P-e_d)) oh2Re_d
template <typename T>
__device__ T rhs_adjoint_point(const View<T> &A, const Coeffs<T> &co, int f, long i, long j, long k) {
  T acc = T(0);
  {
    const int c = f;
    const long ei = c == 0, ej = c == 1, ek = c == 2;
    const T m0 = A.M(c, i, j, k);
    if (m0 != T(0)) acc -= m0 * (A.S(c, i + ei, j + ej, k + ek) - A.S(c, i - ei, j - ej, k - ek)) * co.o2h[c];
    const T mm = A.M(c, i - ei, j - ej, k - ek);
    if (mm != T(0)) acc -= mm * A.S(c, i - ei, j - ej, k - ek) * co.o2h[c];
    const T mp = A.M(c, i + ei, j + ej, k + ek);
    if (mp != T(0)) acc += mp * A.S(c, i + ei, j + ej, k + ek) * co.o2h[c];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const long di = d == 0, dj = d == 1, dk = d == 2;
      const T mdm = A.M(c, i - di, j - dj, k - dk);
      const T mdp = A.M(c, i + di, j + dj, k + dk);
      if (d != c) {
        if (mdm != T(0)) acc -= mdm * avg_dc(A, d, c, i - di, j - dj, k - dk) * co.o8h[d];
        if (mdp != T(0)) acc += mdp * avg_dc(A, d, c, i + di, j + dj, k + dk) * co.o8h[d];
      }
      acc += (mdp - T(2) * m0 + mdm) * co.oh2Re[d];
    }
  }
  // R_c for c != f reads V_f through Avg_{f,c}(P) at P in {Q, Q-e_f, Q+e_c, Q+e_c-e_f}.
  const long di = f == 0, dj = f == 1, dk = f == 2;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (c == f) continue;
    const long ci = c == 0, cj = c == 1, ck = c == 2;
    const long P[4][3] = {{i, j, k},
                          {i - di, j - dj, k - dk},
                          {i + ci, j + cj, k + ck},
                          {i + ci - di, j + cj - dj, k + ck - dk}};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const T m = A.M(c, P[r][0], P[r][1], P[r][2]);
      if (m == T(0)) continue;
      const T dv = A.S(c, P[r][0] + di, P[r][1] + dj, P[r][2] + dk) - A.S(c, P[r][0] - di, P[r][1] - dj, P[r][2] - dk);
      acc -= m * dv * co.o8h[f];
    }
  }
  return acc;
}

// lam_f += (R'(V)^T mu)_f on every point of the three fields.
template <typename T>
__global__ void rhs_adjoint_kernel(View<T> A, Coeffs<T> co, T *l0, T *l1, T *l2) {
  const long i = blockIdx.x * blockDim.x + threadIdx.x;
  const long j = blockIdx.y * blockDim.y + threadIdx.y;
  const long k = blockIdx.z;
  T *lam[3] = {l0, l1, l2};
  const long q = A.g.idx(i, j, k);
#pragma unroll 1
  for (int f = 0; f < 3; ++f) {
    if (i >= A.g.ext(f, 0) || j >= A.g.ext(f, 1) || k >= A.g.ext(f, 2)) continue;
    lam[f][q] += rhs_adjoint_point(A, co, f, i, j, k);
  }
}

// out(r) = (add(r) + scale (G^T mu)(r)) / (weighted ? W(r) : 1) on the pressure
// extents, (G^T mu)(r) = sum_c oh_c (mu_c(r) [r interior of c] - mu_c(r+e_c) [r+e_c interior of c]).
// out may alias add.
template <typename T>
__global__ void grad_adjoint_kernel(Geometry g, T *out, const T *add, const T *m0, const T *m1, const T *m2,
                                    T scale, int weighted) {
  const long i = blockIdx.x * blockDim.x + threadIdx.x;
  const long j = blockIdx.y * blockDim.y + threadIdx.y;
  const long k = blockIdx.z;
  if (i >= g.E[0] || j >= g.E[1]) return;
  const T *mu[3] = {m0, m1, m2};
  T acc = T(0);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const long ei = c == 0, ej = c == 1, ek = c == 2;
    T a = interior(g, c, i, j, k) ? mu[c][g.idx(i, j, k)] : T(0);
    if (interior(g, c, i + ei, j + ej, k + ek)) a -= mu[c][g.idx(i + ei, j + ej, k + ek)];
    acc += a * T(g.oh[c]);
  }
  const long q = g.idx(i, j, k);
  T v = scale * acc;
  if (add) v += add[q];
  if (weighted) v = T((double)v / trap_weight(g, i, j, k));
  out[q] = v;
}

// out_c(q) = in_c(q) + scale (D^T (W rho))_c(q), (D^T r)_c(q) = oh_c (r(q-e_c) - r(q)),
// r taken as zero off the owner block. out may alias in.
template <typename T>
__global__ void div_adjoint_kernel(Geometry g, T *o0, T *o1, T *o2, const T *i0, const T *i1, const T *i2,
                                   const T *rho, T scale) {
  const long i = blockIdx.x * blockDim.x + threadIdx.x;
  const long j = blockIdx.y * blockDim.y + threadIdx.y;
  const long k = blockIdx.z;
  T *out[3] = {o0, o1, o2};
  const T *in[3] = {i0, i1, i2};
  const T r0 = owner(g, i, j, k) ? T((double)rho[g.idx(i, j, k)] * trap_weight(g, i, j, k)) : T(0);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (i >= g.ext(c, 0) || j >= g.ext(c, 1) || k >= g.ext(c, 2)) continue;
    const long ei = c == 0, ej = c == 1, ek = c == 2;
    T rm = T(0);
    if (owner(g, i - ei, j - ej, k - ek))
      rm = T((double)rho[g.idx(i - ei, j - ej, k - ek)] * trap_weight(g, i - ei, j - ej, k - ek));
    const long q = g.idx(i, j, k);
    out[c][q] = in[c][q] + scale * (rm - r0) * T(g.oh[c]);
  }
}

// Adjoint of one periodic copy along axis d (src/StaggeredTensor.cpp:221-257):
// forward a[0] = a[E-2], a[E-1] = a[1]; adjoint lam[1] += lam[E-1], lam[E-2] += lam[0],
// then both ghosts cleared.
template <typename T>
__global__ void periodic_adjoint_kernel(Geometry g, T *f0, T *f1, T *f2, int d, int scalar) {
  const int c = blockIdx.z;
  T *f = c == 0 ? f0 : (c == 1 ? f1 : f2);
  if (!f) return;
  const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
  auto ext = [&](int ax) { return scalar ? g.E[ax] : g.ext(c, ax); };
  const long pa = blockIdx.x * blockDim.x + threadIdx.x;
  const long pb = blockIdx.y * blockDim.y + threadIdx.y;
  if (pa >= ext(a) || pb >= ext(b)) return;
  const int E = ext(d);
  long p[4][3];
  const long dv[4] = {0, 1, E - 2, E - 1};
  for (int r = 0; r < 4; ++r) {
    p[r][a] = pa;
    p[r][b] = pb;
    p[r][d] = dv[r];
  }
  const long q0 = g.idx(p[0][0], p[0][1], p[0][2]), q1 = g.idx(p[1][0], p[1][1], p[1][2]);
  const long qm2 = g.idx(p[2][0], p[2][1], p[2][2]), qm1 = g.idx(p[3][0], p[3][1], p[3][2]);
  f[q1] += f[qm1];
  f[qm1] = T(0);
  f[qm2] += f[q0];
  f[q0] = T(0);
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

// Split of the adjoint of one stage's pre-projection set X (lx, zero off the
// interior) on the interior points:
//   mu   = a lx + b pend      (adjoint weights of this stage's R)
//   pend = a2 lx              (when write_pend: the share of an earlier R)
// and, when tab is given, acc += sum mu_c F_c with F the Taylor-Green
// body-force pattern (sin x cos y cos z, -cos x sin y cos z, 0).
template <typename T>
__global__ void split_kernel(Geometry g, T *m0, T *m1, T *m2, T *p0, T *p1, T *p2, const T *x0, const T *x1,
                             const T *x2, T a, T b, T a2, int write_pend, const T *tab, int maxE, double *acc) {
  const long i = blockIdx.x * blockDim.x + threadIdx.x;
  const long j = blockIdx.y * blockDim.y + threadIdx.y;
  const long k = blockIdx.z;
  T *mu[3] = {m0, m1, m2}, *pend[3] = {p0, p1, p2};
  const T *lx[3] = {x0, x1, x2};
  const long q = g.idx(i, j, k);
  double f = 0.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (!interior(g, c, i, j, k)) continue;
    const T x = lx[c][q];
    T m = a * x;
    if (b != T(0)) m += b * pend[c][q];
    mu[c][q] = m;
    if (write_pend) pend[c][q] = a2 * x;
    if (tab && c < 2) {
      auto S = [&](int ax, int face, long n) { return (double)tab[((ax * 2 + face) * 2 + 0) * maxE + n]; };
      auto C = [&](int ax, int face, long n) { return (double)tab[((ax * 2 + face) * 2 + 1) * maxE + n]; };
      if (c == 0)
        f += (double)m * (S(0, 1, i) * C(1, 0, j) * C(2, 0, k));
      else
        f -= (double)m * (C(0, 0, i) * S(1, 1, j) * C(2, 0, k));
    }
  }
  if (!tab) return;
  for (int o = 16; o > 0; o >>= 1) f += __shfl_down_sync(0xffffffffu, f, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(acc, f);
}

// Kinetic energy in an axis-aligned box at the staggered points:
//   L = 1/2 vol sum_c sum_{q interior of c, position in box} u_c(q)^2
// lam_c(q) = vol u_c(q) there and 0 on every other point; acc += L.
template <typename T>
__global__ void ke_seed_kernel(Geometry g, const T *u0, const T *u1, const T *u2, T *l0, T *l1, T *l2, double x0,
                               double x1, double y0, double y1, double z0, double z1, double *acc) {
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
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(acc, a);
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
  static void rhs_adjoint(const Geometry &g, T *const lam[3], const T *const mu[3], const T *const V[3],
                          cudaStream_t s, long long *cnt) {
    adj::View<T> A{g, {mu[0], mu[1], mu[2]}, {V[0], V[1], V[2]}};
    adj::rhs_adjoint_kernel<T><<<box_grid(g), dim3(32, 8), 0, s>>>(A, coeffs(g), lam[0], lam[1], lam[2]);
    ++*cnt;
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
    for (int d = 2; d >= 0; --d) {
      if (!g.periodic[d]) continue;
      adj::periodic_adjoint_kernel<T><<<dim3(adj::cdiv_u(mx, 32), adj::cdiv_u(mx, 8), 3), dim3(32, 8), 0, s>>>(
          g, f[0], f[1], f[2], d, 0);
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
    for (int d = 2; d >= 0; --d) {
      if (!g.periodic[d]) continue;
      adj::periodic_adjoint_kernel<T><<<dim3(adj::cdiv_u(mx, 32), adj::cdiv_u(mx, 8), 1), dim3(32, 8), 0, s>>>(
          g, f, nullptr, nullptr, d, 1);
      ++*cnt;
    }
  }
  static void split(const Geometry &g, T *const mu[3], T *const pend[3], const T *const lx[3], double a, double b,
                    double a2, bool write_pend, const T *tab, int maxE, double *acc, cudaStream_t s,
                    long long *cnt) {
    adj::split_kernel<T><<<box_grid(g), dim3(32, 8), 0, s>>>(g, mu[0], mu[1], mu[2], pend[0], pend[1], pend[2],
                                                             lx[0], lx[1], lx[2], T(a), T(b), T(a2),
                                                             write_pend ? 1 : 0, tab, maxE, acc);
    ++*cnt;
  }
  static void ke_seed(const Geometry &g, const T *const u[3], T *const lam[3], const double box[6], double *acc,
                      cudaStream_t s, long long *cnt) {
    adj::ke_seed_kernel<T><<<box_grid(g), dim3(32, 8), 0, s>>>(g, u[0], u[1], u[2], lam[0], lam[1], lam[2], box[0],
                                                               box[1], box[2], box[3], box[4], box[5], acc);
    ++*cnt;
  }
};

}  // namespace mifgpu
