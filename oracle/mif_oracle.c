/*
 * Plain-C restatement of the reference's time step — TEST INFRASTRUCTURE ONLY.
 * See mif_oracle.h for scope. Every function cites the reference lines it
 * restates; expressions keep the reference's evaluation order so that the
 * same compiler flags give the same bits.
 */
#include "mif_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "manufactured.h"
#include "r2r.h"

typedef struct {
  long e[3];
  double *a;
} fld;

#define AT(f, i, j, k) ((f)->a[(long)(i) + (f)->e[0] * ((long)(j) + (f)->e[1] * (long)(k))])

typedef struct {
  mif_oracle_params prm;
  int forcing;
  /* Sensitivity probe (not reference behaviour): every forcing value is
   * multiplied by 1 + forcing_noise * r, r in [-1, 1) a hash of the point,
   * the component and forcing_seed. 0 (the default) leaves the restatement
   * bit-identical to the reference. */
  double forcing_noise;
  unsigned forcing_seed;
  /* src/Constants.cpp:58-94 with one rank. */
  double dt, h[3], o2h[3], o8h[3], oh2Re[3], h_2[3], oh[3];
  long E[3];    /* Nx, Ny, Nz */
  long Es[3];   /* Nx_staggered, Ny_staggered, Nz_staggered */
  long base[3]; /* base_i, base_j, base_k */
  long np[3];   /* Poisson points per axis, src/PressureSolverStructures.cpp:15-17 */
  fld vel[3][3];
  fld p, phi;
  double *lam[3];
  double *line;
} St;

static void fld_init(fld *f, long ex, long ey, long ez) {
  f->e[0] = ex, f->e[1] = ey, f->e[2] = ez;
  f->a = (double *)calloc((size_t)(ex * ey * ez), sizeof(double));
}

static fld *field(St *s, int id) {
  if (id >= 0 && id < 9) return &s->vel[id / 3][id % 3];
  if (id == 9) return &s->p;
  if (id == 10) return &s->phi;
  return NULL;
}

/* Sampling positions, src/StaggeredTensor.h:99-104 and include/VelocityTensor.h:16-78:
 * unstaggered node i of axis d, and the face staggered half a cell back. */
static inline double node(const St *s, int d, long i) { return s->prm.origin[d] + s->h[d] * (double)(s->base[d] + i); }
static inline double face(const St *s, int d, long i) { return node(s, d, i) - s->h_2[d]; }

/* Exact value of component c at the sampling point of field c's index (i,j,k). */
static inline double exact_at(const St *s, int c, double t, long i, long j, long k) {
  const double x = c == 0 ? face(s, 0, i) : node(s, 0, i);
  const double y = c == 1 ? face(s, 1, j) : node(s, 1, j);
  const double z = c == 2 ? face(s, 2, k) : node(s, 2, k);
  return mf_eval(s->prm.exact_kind, c, t, x, y, z, s->prm.Re);
}

static inline double eval_kind(const St *s, int kind_fn, int c, double t, double x, double y, double z) {
  /* kind_fn 0: exact velocity; 1: exact pressure gradient. */
  if (kind_fn == 0) return mf_eval(s->prm.exact_kind, c, t, x, y, z, s->prm.Re);
  return mf_pressure_gradient(s->prm.exact_kind, c, t, x, y, z, s->prm.Re);
}

void *mif_oracle_create(const mif_oracle_params *p) {
  St *s = (St *)calloc(1, sizeof(St));
  s->prm = *p;
  s->dt = p->dt / 1u; /* final_time / num_time_steps with one step */
  for (int d = 0; d < 3; ++d) {
    const int per = p->periodic[d] != 0;
    s->h[d] = p->size[d] / (double)(p->n_global[d] - 1);
    s->o2h[d] = 1 / (2 * s->h[d]);
    s->o8h[d] = 1 / (8 * s->h[d]);
    s->oh2Re[d] = 1 / (p->Re * s->h[d] * s->h[d]);
    s->h_2[d] = s->h[d] / 2;
    s->oh[d] = 1 / s->h[d];
    s->E[d] = per ? p->n_global[d] + 1 : p->n_global[d];
    s->base[d] = per ? -1 : 0;
    s->np[d] = p->n_global[d] - (per ? 1 : 0);
  }
  /* src/Constants.cpp:86-88: with one rank the y and z staggered extents
   * always gain a point; x only when not periodic. */
  s->Es[0] = p->periodic[0] ? s->E[0] : s->E[0] + 1;
  s->Es[1] = s->E[1] + 1;
  s->Es[2] = s->E[2] + 1;
  for (int b = 0; b < 3; ++b) {
    fld_init(&s->vel[b][0], s->Es[0], s->E[1], s->E[2]);
    fld_init(&s->vel[b][1], s->E[0], s->Es[1], s->E[2]);
    fld_init(&s->vel[b][2], s->E[0], s->E[1], s->Es[2]);
  }
  fld_init(&s->p, s->E[0], s->E[1], s->E[2]);
  fld_init(&s->phi, s->E[0], s->E[1], s->E[2]);
  /* Eigenvalues, src/PressureSolverStructures.cpp:5-11. */
  long lmax = 1;
  for (int d = 0; d < 3; ++d) {
    const long N = s->np[d];
    s->lam[d] = (double *)malloc(sizeof(double) * (size_t)N);
    for (long i = 0; i < N; ++i) {
      const size_t index = (size_t)i, Ns = (size_t)N;
      s->lam[d][i] = p->periodic[d] ? 2.0 * (cos(2.0 * M_PI * index / Ns) - 1.0) / (s->h[d] * s->h[d])
                                    : 2.0 * (cos(M_PI * index / (Ns - 1)) - 1.0) / (s->h[d] * s->h[d]);
    }
    if (N > lmax) lmax = N;
  }
  s->line = (double *)malloc(sizeof(double) * (size_t)lmax);
  return s;
}

void mif_oracle_destroy(void *h) {
  St *s = (St *)h;
  if (!s) return;
  for (int b = 0; b < 3; ++b)
    for (int c = 0; c < 3; ++c) free(s->vel[b][c].a);
  free(s->p.a);
  free(s->phi.a);
  for (int d = 0; d < 3; ++d) free(s->lam[d]);
  free(s->line);
  free(s);
}

int mif_oracle_set_forcing(void *h, int forcing) {
  ((St *)h)->forcing = forcing;
  return 0;
}

int mif_oracle_set_forcing_noise(void *h, double rel, unsigned seed) {
  ((St *)h)->forcing_noise = rel;
  ((St *)h)->forcing_seed = seed;
  return 0;
}

/* r in [-1, 1) from a 32-bit integer hash (lowbias32) of point, component, seed. */
static double probe_noise(const St *s, int c, long i, long j, long k) {
  unsigned x = (unsigned)(i + s->Es[0] * (j + s->Es[1] * k)) * 3u + (unsigned)c;
  x ^= s->forcing_seed * 0x9e3779b9u;
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return (double)x / 2147483648.0 - 1.0;
}

int mif_oracle_extent(void *h, int id, long out[3]) {
  fld *f = field((St *)h, id);
  if (!f) return -1;
  for (int d = 0; d < 3; ++d) out[d] = f->e[d];
  return 0;
}

int mif_oracle_set(void *h, int id, const double *data) {
  fld *f = field((St *)h, id);
  if (!f) return -1;
  memcpy(f->a, data, sizeof(double) * (size_t)(f->e[0] * f->e[1] * f->e[2]));
  return 0;
}

int mif_oracle_get(void *h, int id, double *data) {
  fld *f = field((St *)h, id);
  if (!f) return -1;
  memcpy(data, f->a, sizeof(double) * (size_t)(f->e[0] * f->e[1] * f->e[2]));
  return 0;
}

/* src/StaggeredTensor.cpp:205-219 with the staggered sampling of each component. */
int mif_oracle_set_exact_velocity(void *h, int set, double t, int include_border) {
  St *s = (St *)h;
  for (int c = 0; c < 3; ++c) {
    fld *f = &s->vel[set][c];
    const long lo = include_border ? 0 : 1;
    for (long k = lo; k < f->e[2] - lo; ++k)
      for (long j = lo; j < f->e[1] - lo; ++j)
        for (long i = lo; i < f->e[0] - lo; ++i) AT(f, i, j, k) = exact_at(s, c, t, i, j, k);
  }
  return 0;
}

int mif_oracle_set_exact_pressure(void *h, double t) {
  St *s = (St *)h;
  fld *f = &s->p;
  for (long k = 0; k < f->e[2]; ++k)
    for (long j = 0; j < f->e[1]; ++j)
      for (long i = 0; i < f->e[0]; ++i)
        AT(f, i, j, k) = mf_eval(s->prm.exact_kind, 3, t, node(s, 0, i), node(s, 1, j), node(s, 2, k), s->prm.Re);
  return 0;
}

/* ---- Momentum right-hand side, include/MomentumEquation.h:42-255 (OPT_CPU_CACHE branch) ---- */

static inline double rhs_u(const St *s, fld *const V[3], long i, long j, long k) {
  const fld *u = V[0], *v = V[1], *w = V[2];
  const double u13 = AT(u, i - 1, j, k), u11 = AT(u, i, j - 1, k), u5 = AT(u, i, j, k - 1), u14 = AT(u, i, j, k),
               u23 = AT(u, i, j, k + 1), u17 = AT(u, i, j + 1, k), u15 = AT(u, i + 1, j, k);
  const double v13 = AT(v, i - 1, j, k), v16 = AT(v, i - 1, j + 1, k), v14 = AT(v, i, j, k), v17 = AT(v, i, j + 1, k);
  const double w13 = AT(w, i - 1, j, k), w22 = AT(w, i - 1, j, k + 1), w14 = AT(w, i, j, k), w23 = AT(w, i, j, k + 1);
  const double conv = -u14 * (u15 - u13) * s->o2h[0] - (v17 + v14 + v16 + v13) * (u17 - u11) * s->o8h[1] -
                      (w23 + w14 + w22 + w13) * (u23 - u5) * s->o8h[2];
  const double diff = (u15 - 2 * u14 + u13) * s->oh2Re[0] + (u17 - 2 * u14 + u11) * s->oh2Re[1] +
                      (u23 - 2 * u14 + u5) * s->oh2Re[2];
  return conv + diff;
}

static inline double rhs_v(const St *s, fld *const V[3], long i, long j, long k) {
  const fld *u = V[0], *v = V[1], *w = V[2];
  const double u11 = AT(u, i, j - 1, k), u14 = AT(u, i, j, k), u12 = AT(u, i + 1, j - 1, k), u15 = AT(u, i + 1, j, k);
  const double v13 = AT(v, i - 1, j, k), v11 = AT(v, i, j - 1, k), v5 = AT(v, i, j, k - 1), v14 = AT(v, i, j, k),
               v23 = AT(v, i, j, k + 1), v17 = AT(v, i, j + 1, k), v15 = AT(v, i + 1, j, k);
  const double w11 = AT(w, i, j - 1, k), w20 = AT(w, i, j - 1, k + 1), w14 = AT(w, i, j, k), w23 = AT(w, i, j, k + 1);
  const double conv = -(u15 + u14 + u12 + u11) * (v15 - v13) * s->o8h[0] - v14 * (v17 - v11) * s->o2h[1] -
                      (w23 + w14 + w20 + w11) * (v23 - v5) * s->o8h[2];
  const double diff = (v15 - 2 * v14 + v13) * s->oh2Re[0] + (v17 - 2 * v14 + v11) * s->oh2Re[1] +
                      (v23 - 2 * v14 + v5) * s->oh2Re[2];
  return conv + diff;
}

static inline double rhs_w(const St *s, fld *const V[3], long i, long j, long k) {
  const fld *u = V[0], *v = V[1], *w = V[2];
  const double u5 = AT(u, i, j, k - 1), u14 = AT(u, i, j, k), u6 = AT(u, i + 1, j, k - 1), u15 = AT(u, i + 1, j, k);
  const double v5 = AT(v, i, j, k - 1), v14 = AT(v, i, j, k), v8 = AT(v, i, j + 1, k - 1), v17 = AT(v, i, j + 1, k);
  const double w13 = AT(w, i - 1, j, k), w11 = AT(w, i, j - 1, k), w5 = AT(w, i, j, k - 1), w14 = AT(w, i, j, k),
               w23 = AT(w, i, j, k + 1), w17 = AT(w, i, j + 1, k), w15 = AT(w, i + 1, j, k);
  const double conv = -(u15 + u14 + u6 + u5) * (w15 - w13) * s->o8h[0] - (v17 + v14 + v8 + v5) * (w17 - w11) * s->o8h[1] -
                      w14 * (w23 - w5) * s->o2h[2];
  const double diff = (w15 - 2 * w14 + w13) * s->oh2Re[0] + (w17 - 2 * w14 + w11) * s->oh2Re[1] +
                      (w23 - 2 * w14 + w5) * s->oh2Re[2];
  return conv + diff;
}

/* Momentum RHS of component c, plus the forcing at the component's staggered
 * point when enabled (include/MomentumEquationForcing.h:10-32). */
static inline double rhs(const St *s, int c, fld *const V[3], long i, long j, long k, double t) {
  double r = c == 0 ? rhs_u(s, V, i, j, k) : (c == 1 ? rhs_v(s, V, i, j, k) : rhs_w(s, V, i, j, k));
  if (s->forcing) {
    const double x = c == 0 ? face(s, 0, i) : node(s, 0, i);
    const double y = c == 1 ? face(s, 1, j) : node(s, 1, j);
    const double z = c == 2 ? face(s, 2, k) : node(s, 2, k);
    double f = mf_forcing(s->prm.exact_kind, c, t, x, y, z, s->prm.Re, s->forcing == 2);
    if (s->forcing_noise != 0.0) f = f * (1.0 + s->forcing_noise * probe_noise(s, c, i, j, k));
    r = r + f;
  }
  return r;
}

/* include/PressureGradient.h:9-24 */
static inline double grad(const St *s, int c, const fld *p, long i, long j, long k) {
  if (c == 0) return (AT(p, i, j, k) - AT(p, i - 1, j, k)) * s->oh[0];
  if (c == 1) return (AT(p, i, j, k) - AT(p, i, j - 1, k)) * s->oh[1];
  return (AT(p, i, j, k) - AT(p, i, j, k - 1)) * s->oh[2];
}

#define INTERIOR(f) \
  for (long k = 1; k < (f)->e[2] - 1; ++k) \
    for (long j = 1; j < (f)->e[1] - 1; ++j) \
      for (long i = 1; i < (f)->e[0] - 1; ++i)

/* ---- Stage updates of the projection step, src/Timestep.cpp:10-54 ---- */

static void stage_y2(St *s, double t) {
  fld *V0[3] = {&s->vel[0][0], &s->vel[0][1], &s->vel[0][2]};
  const double dt = s->dt, a1 = 64.0 / 120.0 * dt, b = a1;
  for (int c = 0; c < 3; ++c) {
    fld *u = V0[c], *b1 = &s->vel[1][c], *b2 = &s->vel[2][c];
    INTERIOR(u) {
      const double r = rhs(s, c, V0, i, j, k, t);
      const double g = grad(s, c, &s->p, i, j, k);
      AT(b1, i, j, k) = AT(u, i, j, k) + a1 * r - b * g;
      AT(b2, i, j, k) = r;
    }
  }
}

static void stage_y3(St *s, double t) {
  fld *V1[3] = {&s->vel[1][0], &s->vel[1][1], &s->vel[1][2]};
  const double dt = s->dt, a1 = -34.0 / 120.0 * dt, a2 = 50.0 / 120.0 * dt, b = a1 + a2;
  for (int c = 0; c < 3; ++c) {
    fld *u = &s->vel[0][c], *b1 = V1[c], *b2 = &s->vel[2][c];
    INTERIOR(b2) {
      const double r1 = AT(b2, i, j, k);
      const double r2 = rhs(s, c, V1, i, j, k, t);
      const double r2s = a2 * r2;
      const double g = grad(s, c, &s->p, i, j, k);
      AT(b2, i, j, k) = AT(b1, i, j, k) + a1 * r1 + r2s - b * g;
      AT(u, i, j, k) = r2s;
    }
  }
}

static void stage_ustar(St *s, double t) {
  fld *V2[3] = {&s->vel[2][0], &s->vel[2][1], &s->vel[2][2]};
  const double dt = s->dt, a2 = -50.0 / 120.0 * dt, a3 = 90.0 / 120.0 * dt, b = a2 + a3;
  for (int c = 0; c < 3; ++c) {
    fld *u = &s->vel[0][c], *b2 = V2[c];
    INTERIOR(u) {
      const double r2s = -AT(u, i, j, k);
      const double r3 = rhs(s, c, V2, i, j, k, t);
      const double g = grad(s, c, &s->p, i, j, k);
      AT(u, i, j, k) = AT(b2, i, j, k) + r2s + a3 * r3 - b * g;
    }
  }
}

/* ---- Boundary fill, src/VelocityTensor.cpp:36-233 ---- */

/* src/StaggeredTensor.cpp:221-257 */
static void periodic_fill(const St *s, fld *f) {
  const long ex = f->e[0], ey = f->e[1], ez = f->e[2];
  if (s->prm.periodic[0])
    for (long k = 0; k < ez; ++k)
      for (long j = 0; j < ey; ++j) {
        AT(f, 0, j, k) = AT(f, ex - 2, j, k);
        AT(f, ex - 1, j, k) = AT(f, 1, j, k);
      }
  if (s->prm.periodic[1])
    for (long k = 0; k < ez; ++k)
      for (long i = 0; i < ex; ++i) {
        AT(f, i, 0, k) = AT(f, i, ey - 2, k);
        AT(f, i, ey - 1, k) = AT(f, i, 1, k);
      }
  if (s->prm.periodic[2])
    for (long j = 0; j < ey; ++j)
      for (long i = 0; i < ex; ++i) {
        AT(f, i, j, 0) = AT(f, i, j, ez - 2);
        AT(f, i, j, ez - 1) = AT(f, i, j, 1);
      }
}

/* Dirichlet faces then periodic copy for one velocity set; fn selects the
 * function family (0 exact velocity, 1 exact pressure gradient). */
static void apply_bc_fn(St *s, fld *const V[3], double t, int fn) {
  const int *per = s->prm.periodic;
  for (int c = 0; c < 3; ++c) {
    fld *f = V[c];
    const long ex = f->e[0], ey = f->e[1], ez = f->e[2];
#define EV(cc, x, y, z) eval_kind(s, fn, cc, t, x, y, z)
/* staggered sampling of component cc at index (i,j,k) */
#define SX(cc, i) ((cc) == 0 ? face(s, 0, i) : node(s, 0, i))
#define SY(cc, j) ((cc) == 1 ? face(s, 1, j) : node(s, 1, j))
#define SZ(cc, k) ((cc) == 2 ? face(s, 2, k) : node(s, 2, k))
#define EVS(cc, i, j, k) EV(cc, SX(cc, i), SY(cc, j), SZ(cc, k))
    /* Face 1: z = z_min */
    if (!per[2]) {
      for (long j = 0; j < ey; ++j)
        for (long i = 0; i < ex; ++i) {
          if (c == 2) {
            const double wb = EV(2, node(s, 0, i), node(s, 1, j), node(s, 2, 0));
            const double du = (EVS(0, i + 1, j, 0) - EVS(0, i, j, 0)) * s->oh[0];
            const double dv = (EVS(1, i, j + 1, 0) - EVS(1, i, j, 0)) * s->oh[1];
            AT(f, i, j, 0) = wb + s->h_2[2] * (du + dv);
          } else {
            AT(f, i, j, 0) = EVS(c, i, j, 0);
          }
        }
    }
    /* Face 2: z = z_max */
    if (!per[2]) {
      const long K = s->E[2] - 1;
      for (long j = 0; j < ey; ++j)
        for (long i = 0; i < ex; ++i) {
          if (c == 2) {
            const double wb = EV(2, node(s, 0, i), node(s, 1, j), node(s, 2, K));
            const double du = (EVS(0, i + 1, j, K) - EVS(0, i, j, K)) * s->oh[0];
            const double dv = (EVS(1, i, j + 1, K) - EVS(1, i, j, K)) * s->oh[1];
            AT(f, i, j, s->Es[2] - 1) = wb - s->h_2[2] * (du + dv);
          } else {
            AT(f, i, j, K) = EVS(c, i, j, K);
          }
        }
    }
    /* Face 3: y = y_min */
    if (!per[1]) {
      for (long k = 0; k < ez; ++k)
        for (long i = 0; i < ex; ++i) {
          if (c == 1) {
            const double vb = EV(1, node(s, 0, i), node(s, 1, 0), node(s, 2, k));
            const double du = (EVS(0, i + 1, 0, k) - EVS(0, i, 0, k)) * s->oh[0];
            const double dw = (EVS(2, i, 0, k + 1) - EVS(2, i, 0, k)) * s->oh[2];
            AT(f, i, 0, k) = vb + s->h_2[1] * (du + dw);
          } else {
            AT(f, i, 0, k) = EVS(c, i, 0, k);
          }
        }
    }
    /* Face 4: y = y_max */
    if (!per[1]) {
      const long J = s->E[1] - 1;
      for (long k = 0; k < ez; ++k)
        for (long i = 0; i < ex; ++i) {
          if (c == 1) {
            const double vb = EV(1, node(s, 0, i), node(s, 1, J), node(s, 2, k));
            const double du = (EVS(0, i + 1, J, k) - EVS(0, i, J, k)) * s->oh[0];
            const double dw = (EVS(2, i, J, k + 1) - EVS(2, i, J, k)) * s->oh[2];
            AT(f, i, s->Es[1] - 1, k) = vb - s->h_2[1] * (du + dw);
          } else {
            AT(f, i, J, k) = EVS(c, i, J, k);
          }
        }
    }
    /* Face 5: x = x_min */
    if (!per[0]) {
      for (long k = 0; k < ez; ++k)
        for (long j = 0; j < ey; ++j) {
          if (c == 0) {
            const double ub = EV(0, node(s, 0, 0), node(s, 1, j), node(s, 2, k));
            const double dv = (EVS(1, 0, j + 1, k) - EVS(1, 0, j, k)) * s->oh[1];
            const double dw = (EVS(2, 0, j, k + 1) - EVS(2, 0, j, k)) * s->oh[2];
            AT(f, 0, j, k) = ub + s->h_2[0] * (dv + dw);
          } else {
            AT(f, 0, j, k) = EVS(c, 0, j, k);
          }
        }
    }
    /* Face 6: x = x_max */
    if (!per[0]) {
      const long I = s->E[0] - 1;
      for (long k = 0; k < ez; ++k)
        for (long j = 0; j < ey; ++j) {
          if (c == 0) {
            const double ub = EV(0, node(s, 0, s->prm.n_global[0] - 1), node(s, 1, j), node(s, 2, k));
            const double dv = (EVS(1, I, j + 1, k) - EVS(1, I, j, k)) * s->oh[1];
            const double dw = (EVS(2, I, j, k + 1) - EVS(2, I, j, k)) * s->oh[2];
            AT(f, s->Es[0] - 1, j, k) = ub - s->h_2[0] * (dv + dw);
          } else {
            AT(f, I, j, k) = EVS(c, I, j, k);
          }
        }
    }
#undef EV
#undef SX
#undef SY
#undef SZ
#undef EVS
    periodic_fill(s, f);
  }
}

int mif_oracle_apply_bc(void *h, int set, double t) {
  St *s = (St *)h;
  fld *V[3] = {&s->vel[set][0], &s->vel[set][1], &s->vel[set][2]};
  apply_bc_fn(s, V, t, 0);
  return 0;
}

/* ---- Poisson solve, src/PressureEquation.cpp:10-274 ---- */

/* Owner range of the pressure field along axis d, include/StaggeredTensorMacros.h:41-83. */
static inline long own_lo(const St *s, int d) { return s->prm.periodic[d] ? 1 : 0; }

/* src/PressureEquation.cpp:59-61 with include/VelocityDivergence.h:9-20 */
static void compute_rhs(St *s, fld *const V[3], double dt) {
  fld *r = &s->phi;
  const long i0 = own_lo(s, 0), j0 = own_lo(s, 1), k0 = own_lo(s, 2);
  for (long k = k0; k < k0 + s->np[2]; ++k)
    for (long j = j0; j < j0 + s->np[1]; ++j)
      for (long i = i0; i < i0 + s->np[0]; ++i) {
        const double du = (AT(V[0], i + 1, j, k) - AT(V[0], i, j, k)) * s->oh[0];
        const double dv = (AT(V[1], i, j + 1, k) - AT(V[1], i, j, k)) * s->oh[1];
        const double dw = (AT(V[2], i, j, k + 1) - AT(V[2], i, j, k)) * s->oh[2];
        AT(r, i, j, k) = (du + dv + dw) / dt;
      }
}

/* src/PressureEquation.cpp:10-56 (all axes Neumann) */
static void add_neumann_flux(St *s, double t_a, double t_b) {
  /* g = grad p(t_b) - grad p(t_a), src/VectorFunction.cpp:62-71 */
  fld *r = &s->phi;
  const long ex = r->e[0], ey = r->e[1], ez = r->e[2];
#define G(c, i, j, k)                                                                            \
  (mf_pressure_gradient(s->prm.exact_kind, c, t_b, node(s, 0, i), node(s, 1, j), node(s, 2, k), s->prm.Re) - \
   mf_pressure_gradient(s->prm.exact_kind, c, t_a, node(s, 0, i), node(s, 1, j), node(s, 2, k), s->prm.Re))
  for (long j = 0; j < ey; ++j)
    for (long i = 0; i < ex; ++i) AT(r, i, j, 0) += G(2, i, j, 0) * 2.0 * s->oh[2];
  for (long j = 0; j < ey; ++j)
    for (long i = 0; i < ex; ++i) AT(r, i, j, ez - 1) -= G(2, i, j, ez - 1) * 2.0 * s->oh[2];
  for (long k = 0; k < ez; ++k)
    for (long i = 0; i < ex; ++i) AT(r, i, 0, k) += G(1, i, 0, k) * 2.0 * s->oh[1];
  for (long k = 0; k < ez; ++k)
    for (long i = 0; i < ex; ++i) AT(r, i, ey - 1, k) -= G(1, i, ey - 1, k) * 2.0 * s->oh[1];
  for (long j = 0; j < ey; ++j)
    for (long k = 0; k < ez; ++k) AT(r, 0, j, k) += G(0, 0, j, k) * 2.0 * s->oh[0];
  for (long j = 0; j < ey; ++j)
    for (long k = 0; k < ez; ++k) AT(r, ex - 1, j, k) -= G(0, ex - 1, j, k) * 2.0 * s->oh[0];
#undef G
}

/* One 1-D transform over every line of axis d inside the owner block of phi;
 * norm != 0 divides each output by it (the inverse-direction normalisation). */
static void transform_axis(St *s, int d, int inverse, double norm) {
  fld *f = &s->phi;
  const int kind = s->prm.periodic[d] ? (inverse ? ORACLE_HC2R : ORACLE_R2HC) : ORACLE_REDFT00;
  const long lo[3] = {own_lo(s, 0), own_lo(s, 1), own_lo(s, 2)};
  const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2; /* the two other axes */
  const long stride[3] = {1, f->e[0], f->e[0] * f->e[1]};
  const long n = s->np[d];
  for (long q = 0; q < s->np[b]; ++q)
    for (long r = 0; r < s->np[a]; ++r) {
      const long off = (lo[a] + r) * stride[a] + (lo[b] + q) * stride[b] + lo[d] * stride[d];
      for (long m = 0; m < n; ++m) s->line[m] = f->a[off + m * stride[d]];
      oracle_r2r_1d((int)n, kind, s->line, s->line);
      if (norm != 0.0)
        for (long m = 0; m < n; ++m) s->line[m] /= norm;
      for (long m = 0; m < n; ++m) f->a[off + m * stride[d]] = s->line[m];
    }
}

/* src/PressureEquation.cpp:65-264 restated on the owner block: the reference's
 * pencil transposes (deps/2Decomp_C/Transpose*.cpp) only permute storage, so the
 * same 1-D transforms run on strided lines here. Then the periodic refresh of
 * src/PressureTensor.cpp:21-34. */
static void solve_poisson(St *s) {
  fld *f = &s->phi;
  transform_axis(s, 0, 0, 0.0);
  transform_axis(s, 1, 0, 0.0);
  transform_axis(s, 2, 0, 0.0);
  const long lo[3] = {own_lo(s, 0), own_lo(s, 1), own_lo(s, 2)};
  for (long k = 0; k < s->np[2]; ++k)
    for (long j = 0; j < s->np[1]; ++j)
      for (long i = 0; i < s->np[0]; ++i) {
        const double eig = 1 / (s->lam[0][i] + s->lam[1][j] + s->lam[2][k]);
        AT(f, lo[0] + i, lo[1] + j, lo[2] + k) *= eig;
      }
  AT(f, lo[0], lo[1], lo[2]) = 0;
  const double nz = (double)(s->prm.n_global[2] - 1) * (s->prm.periodic[2] ? 1.0 : 2.0);
  const double ny = (double)(s->prm.n_global[1] - 1) * (s->prm.periodic[1] ? 1.0 : 2.0);
  const double nx = (double)(s->prm.n_global[0] - 1) * (s->prm.periodic[0] ? 1.0 : 2.0);
  transform_axis(s, 2, 1, nz);
  transform_axis(s, 1, 1, ny);
  transform_axis(s, 0, 1, nx);
  periodic_fill(s, f);
}

int mif_oracle_solve_pressure(void *h, int set, double dt) {
  St *s = (St *)h;
  fld *V[3] = {&s->vel[set][0], &s->vel[set][1], &s->vel[set][2]};
  compute_rhs(s, V, dt);
  solve_poisson(s);
  return 0;
}

int mif_oracle_solve_pressure_nhn(void *h, int set, double dt, double t_new, double t_old) {
  St *s = (St *)h;
  fld *V[3] = {&s->vel[set][0], &s->vel[set][1], &s->vel[set][2]};
  compute_rhs(s, V, dt);
  /* src/Timestep.cpp:88-93: get_difference_over_time(new_time, prev_time)
   * evaluates f(prev_time) - f(new_time). */
  add_neumann_flux(s, t_new, t_old);
  solve_poisson(s);
  return 0;
}

/* ---- Pressure accumulation and projection, src/Timestep.cpp:66-81 ---- */

static void update_pressure(St *s) {
  const long n = s->p.e[0] * s->p.e[1] * s->p.e[2];
  for (long q = 0; q < n; ++q) s->p.a[q] += s->phi.a[q];
}

static void project(St *s, int set, double dt_k) {
  for (int c = 0; c < 3; ++c) {
    fld *u = &s->vel[set][c];
    INTERIOR(u) { AT(u, i, j, k) -= grad(s, c, &s->phi, i, j, k) * dt_k; }
  }
}

/* The pair the step runs after each Poisson solve, as one call. */
int mif_oracle_project(void *h, int set, double dt) {
  St *s = (St *)h;
  if (set < 0 || set > 2) return -1;
  update_pressure(s);
  project(s, set, dt);
  return 0;
}

/* src/Timestep.cpp:97-156 */
static void full_step(St *s, double t_n, int nhn) {
  const double dt_1 = 64.0 / 120.0 * s->dt;
  const double time_1 = t_n + dt_1;
  const double dt_2 = 16.0 / 120.0 * s->dt;
  const double time_2 = time_1 + dt_2;
  const double dt_3 = 40.0 / 120.0 * s->dt;
  const double final_time = t_n + s->dt;
  const double dts[3] = {dt_1, dt_2, dt_3};
  const double t_new[3] = {time_1, time_2, final_time};
  const double t_old[3] = {t_n, time_1, time_2};
  const int out_set[3] = {1, 2, 0};
  for (int st = 0; st < 3; ++st) {
    if (st == 0) stage_y2(s, t_n);
    if (st == 1) stage_y3(s, time_1);
    if (st == 2) stage_ustar(s, time_2);
    mif_oracle_apply_bc(s, out_set[st], t_new[st]);
    if (nhn)
      mif_oracle_solve_pressure_nhn(s, out_set[st], dts[st], t_new[st], t_old[st]);
    else
      mif_oracle_solve_pressure(s, out_set[st], dts[st]);
    update_pressure(s);
    project(s, out_set[st], dts[st]);
  }
}

int mif_oracle_timestep(void *h, double t_n) {
  full_step((St *)h, t_n, 0);
  return 0;
}

int mif_oracle_timestep_nhn(void *h, double t_n) {
  full_step((St *)h, t_n, 1);
  return 0;
}

/* ---- Velocity-only step, src/TimestepVelocity.cpp:11-90 (always forced) ---- */

int mif_oracle_timestep_velocity(void *h, double t_n) {
  St *s = (St *)h;
  const int saved = s->forcing;
  s->forcing = 1;
  const double c2 = (8.0 / 15.0), a21 = (8.0 / 15.0), c3 = (2.0 / 3.0), a31 = (1.0 / 4.0), a32 = (5.0 / 12.0),
               b1 = (1.0 / 4.0), b3 = (3.0 / 4.0);
  const double dt = s->dt;
  const double time_1 = t_n + c2 * dt, time_2 = t_n + c3 * dt, final_time = t_n + dt;
  fld *V0[3] = {&s->vel[0][0], &s->vel[0][1], &s->vel[0][2]};
  fld *V1[3] = {&s->vel[1][0], &s->vel[1][1], &s->vel[1][2]};
  for (int c = 0; c < 3; ++c) {
    fld *u = V0[c], *b = V1[c], *r = &s->vel[2][c];
    INTERIOR(u) {
      const double q = rhs(s, c, V0, i, j, k, t_n);
      AT(r, i, j, k) = q;
      AT(b, i, j, k) = AT(u, i, j, k) + dt * a21 * q;
    }
  }
  mif_oracle_apply_bc(s, 1, time_1);
  for (int c = 0; c < 3; ++c) {
    fld *u = V0[c], *r = &s->vel[2][c];
    INTERIOR(u) {
      const double q = AT(r, i, j, k);
      AT(r, i, j, k) = AT(u, i, j, k) + dt * (b1 * q);
      AT(u, i, j, k) = AT(u, i, j, k) + dt * (a31 * q + a32 * rhs(s, c, V1, i, j, k, time_1));
    }
  }
  mif_oracle_apply_bc(s, 0, time_2);
  for (int c = 0; c < 3; ++c) {
    fld *u = V0[c], *b = V1[c], *r = &s->vel[2][c];
    INTERIOR(u) {
      const double q = AT(r, i, j, k);
      AT(b, i, j, k) = q + dt * (b3 * rhs(s, c, V0, i, j, k, time_2));
    }
  }
  mif_oracle_apply_bc(s, 1, final_time);
  /* swap_data, src/VelocityTensor.cpp:13-26 */
  for (int c = 0; c < 3; ++c) {
    double *tmp = s->vel[0][c].a;
    s->vel[0][c].a = s->vel[1][c].a;
    s->vel[1][c].a = tmp;
  }
  s->forcing = saved;
  return 0;
}

/* ---- Error measures, src/Norms.cpp:11-118 and src/PressureEquation.cpp:288-343 ---- */

int mif_oracle_adjust_pressure(void *h, double t) {
  St *s = (St *)h;
  fld *p = &s->p;
  double diff = 0;
  const long lo[3] = {own_lo(s, 0), own_lo(s, 1), own_lo(s, 2)};
  for (long k = lo[2]; k < lo[2] + s->np[2]; ++k)
    for (long j = lo[1]; j < lo[1] + s->np[1]; ++j)
      for (long i = lo[0]; i < lo[0] + s->np[0]; ++i)
        diff += mf_eval(s->prm.exact_kind, 3, t, node(s, 0, i), node(s, 1, j), node(s, 2, k), s->prm.Re) - AT(p, i, j, k);
  diff /= (double)(size_t)(s->np[0] * s->np[1] * s->np[2]);
  for (long k = 0; k < s->E[2]; ++k)
    for (long j = 0; j < s->E[1]; ++j)
      for (long i = 0; i < s->E[0]; ++i) AT(p, i, j, k) += diff;
  return 0;
}

/* L1, L2, Linf of a velocity set interpolated to interior nodes; fn picks the
 * exact family (0 velocity, 1 pressure gradient). */
static void velocity_norms(St *s, fld *const V[3], double t, int fn, double out[3]) {
  double l1 = 0, l2 = 0, li = 0;
  for (long k = 1; k < s->E[2] - 1; ++k) {
    const double z = s->prm.origin[2] + (double)(s->base[2] + k) * s->h[2];
    for (long j = 1; j < s->E[1] - 1; ++j) {
      const double y = s->prm.origin[1] + (double)(s->base[1] + j) * s->h[1];
      for (long i = 1; i < s->E[0] - 1; ++i) {
        const double x = s->prm.origin[0] + (double)(s->base[0] + i) * s->h[0];
        const double iu = (AT(V[0], i, j, k) + AT(V[0], i + 1, j, k)) / 2.0;
        const double iv = (AT(V[1], i, j, k) + AT(V[1], i, j + 1, k)) / 2.0;
        const double iw = (AT(V[2], i, j, k) + AT(V[2], i, j, k + 1)) / 2.0;
        const double eu = eval_kind(s, fn, 0, t, x, y, z) - iu;
        const double ev = eval_kind(s, fn, 1, t, x, y, z) - iv;
        const double ew = eval_kind(s, fn, 2, t, x, y, z) - iw;
        l1 = l1 + sqrt(eu * eu + ev * ev + ew * ew);
        l2 = l2 + eu * eu + ev * ev + ew * ew;
        const double m = fmax(fmax(fabs(eu), fabs(ev)), fabs(ew));
        li = li > m ? li : m;
      }
    }
  }
  out[0] = l1 * s->h[0] * s->h[1] * s->h[2];
  out[1] = sqrt(l2 * s->h[0] * s->h[1] * s->h[2]);
  out[2] = li;
}

int mif_oracle_error_norms(void *h, double t, double out[9]) {
  St *s = (St *)h;
  fld *V0[3] = {&s->vel[0][0], &s->vel[0][1], &s->vel[0][2]};
  velocity_norms(s, V0, t, 0, out);
  double l1 = 0, l2 = 0, li = 0;
  const long lo[3] = {own_lo(s, 0), own_lo(s, 1), own_lo(s, 2)};
  for (long k = lo[2]; k < lo[2] + s->np[2]; ++k)
    for (long j = lo[1]; j < lo[1] + s->np[1]; ++j)
      for (long i = lo[0]; i < lo[0] + s->np[0]; ++i) {
        const double z = s->prm.origin[2] + (double)(s->base[2] + k) * s->h[2];
        const double y = s->prm.origin[1] + (double)(s->base[1] + j) * s->h[1];
        const double x = s->prm.origin[0] + (double)(s->base[0] + i) * s->h[0];
        const double e = mf_eval(s->prm.exact_kind, 3, t, x, y, z, s->prm.Re) - AT(&s->p, i, j, k);
        l1 = l1 + fabs(e);
        l2 = l2 + e * e;
        li = li > fabs(e) ? li : fabs(e);
      }
  out[3] = l1 * s->h[0] * s->h[1] * s->h[2];
  out[4] = sqrt(l2 * s->h[0] * s->h[1] * s->h[2]);
  out[5] = li;
  /* test/full_test.cpp:141-143: gradient of p on staggered points, boundary
   * filled from the exact gradient, then the velocity norms. */
  fld G[3];
  fld_init(&G[0], s->Es[0], s->E[1], s->E[2]);
  fld_init(&G[1], s->E[0], s->Es[1], s->E[2]);
  fld_init(&G[2], s->E[0], s->E[1], s->Es[2]);
  fld *GV[3] = {&G[0], &G[1], &G[2]};
  for (int c = 0; c < 3; ++c) {
    fld *g = GV[c];
    INTERIOR(g) { AT(g, i, j, k) = grad(s, c, &s->p, i, j, k); }
  }
  apply_bc_fn(s, GV, t, 1);
  velocity_norms(s, GV, t, 1, out + 6);
  for (int c = 0; c < 3; ++c) free(G[c].a);
  return 0;
}

/* Point evaluations of the analytic families, for formula checks. */
double mif_oracle_forcing_value(int kind, int comp, double t, double x, double y, double z, double Re, int with_p) {
  return mf_forcing(kind, comp, t, x, y, z, Re, with_p);
}

double mif_oracle_pressure_gradient_value(int kind, int comp, double t, double x, double y, double z, double Re) {
  return mf_pressure_gradient(kind, comp, t, x, y, z, Re);
}
