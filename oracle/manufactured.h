/*
 * Analytic fields used as boundary data, forcing and initial conditions —
 * TEST INFRASTRUCTURE ONLY (oracle side; the CUDA library carries its own
 * device copy of the same formulas).
 *
 * Kinds (the numbering is shared with include/mifgpu.h, MIFGPU_FIELD_*):
 *  0 ZERO     : u = v = w = p = 0 (no-slip walls, periodic boxes).
 *  1 SINCOS   : u = sin x cos y sin z sin t, v = cos x sin y sin z sin t,
 *               w = 2 cos x cos y cos z sin t, p = cos x cos y sin z sin t.
 *               The velocity is the reference's velocity-test solution
 *               (generators/manufsol_velocity.py:55-57).
 *  2 ETHIER   : the exact Navier-Stokes solution of the reference's full-step
 *               test (generators/manufsol.py:35-72, a = pi/4, d = pi/2).
 * Forcing (SINCOS only): f = u_t + (u . grad) u - lap(u)/Re, the momentum
 * residual the reference generates in generators/manufsol_velocity.py:32-50;
 * with_pressure adds grad p so that the projection step reproduces the
 * manufactured pressure as well.
 */
#ifndef ORACLE_MANUFACTURED_H
#define ORACLE_MANUFACTURED_H

#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { MF_ZERO = 0, MF_SINCOS = 1, MF_ETHIER = 2 };

/* comp: 0 = u, 1 = v, 2 = w, 3 = p. */
static inline double mf_eval(int kind, int comp, double t, double x, double y, double z, double Re) {
  if (kind == MF_SINCOS) {
    const double st = sin(t);
    switch (comp) {
      case 0: return sin(x) * cos(y) * sin(z) * st;
      case 1: return cos(x) * sin(y) * sin(z) * st;
      case 2: return 2.0 * cos(x) * cos(y) * cos(z) * st;
      default: return cos(x) * cos(y) * sin(z) * st;
    }
  }
  if (kind == MF_ETHIER) {
    const double a = M_PI / 4.0, d = M_PI / 2.0;
    const double decay = exp(-d * d * t / Re);
    switch (comp) {
      case 0: return -a * (exp(a * x) * sin(a * y + d * z) + exp(a * z) * cos(a * x + d * y)) * decay;
      case 1: return -a * (exp(a * y) * sin(a * z + d * x) + exp(a * x) * cos(a * y + d * z)) * decay;
      case 2: return -a * (exp(a * z) * sin(a * x + d * y) + exp(a * y) * cos(a * z + d * x)) * decay;
      default: {
        const double A = a * x + d * y, B = a * y + d * z, C = a * z + d * x;
        return -a * a / 2.0 *
               (exp(2 * a * x) + exp(2 * a * y) + exp(2 * a * z) + 2 * sin(A) * cos(C) * exp(a * (y + z)) +
                2 * sin(B) * cos(A) * exp(a * (z + x)) + 2 * sin(C) * cos(B) * exp(a * (x + y))) *
               decay * decay;
      }
    }
  }
  return 0.0;
}

/* d p / d x_comp of the kind's pressure (comp 0..2). */
static inline double mf_pressure_gradient(int kind, int comp, double t, double x, double y, double z,
                                          double Re) {
  if (kind == MF_SINCOS) {
    const double st = sin(t);
    switch (comp) {
      case 0: return -sin(x) * cos(y) * sin(z) * st;
      case 1: return -cos(x) * sin(y) * sin(z) * st;
      default: return cos(x) * cos(y) * cos(z) * st;
    }
  }
  if (kind == MF_ETHIER) {
    /* p is invariant under the cyclic map (x,y,z) -> (y,z,x), so the y and z
     * derivatives are the x derivative evaluated at the rotated point. */
    const double a = M_PI / 4.0, d = M_PI / 2.0;
    const double decay2 = exp(-2.0 * d * d * t / Re);
    double X = x, Y = y, Z = z;
    if (comp == 1) X = y, Y = z, Z = x;
    if (comp == 2) X = z, Y = x, Z = y;
    const double A = a * X + d * Y, B = a * Y + d * Z, C = a * Z + d * X;
    const double s = 2 * a * exp(2 * a * X) + 2 * exp(a * (Y + Z)) * (a * cos(A) * cos(C) - d * sin(A) * sin(C)) +
                     2 * a * sin(B) * exp(a * (Z + X)) * (cos(A) - sin(A)) +
                     2 * cos(B) * exp(a * (X + Y)) * (d * cos(C) + a * sin(C));
    return -a * a / 2.0 * s * decay2;
  }
  return 0.0;
}

/* Momentum forcing of the SINCOS solution for component comp. */
static inline double mf_forcing(int kind, int comp, double t, double x, double y, double z, double Re,
                                int with_pressure) {
  if (kind != MF_SINCOS) return 0.0;
  const double sx = sin(x), cx = cos(x), sy = sin(y), cy = cos(y), sz = sin(z), cz = cos(z);
  const double st = sin(t), ct = cos(t);
  double f;
  switch (comp) {
    case 0:
      f = sx * cy * sz * ct + st * st * sx * cx * (cy * cy * sz * sz - sy * sy * sz * sz + 2.0 * cy * cy * cz * cz) +
          3.0 * sx * cy * sz * st / Re;
      if (with_pressure) f += -sx * cy * sz * st;
      return f;
    case 1:
      f = cx * sy * sz * ct + st * st * sy * cy * (cx * cx * sz * sz - sx * sx * sz * sz + 2.0 * cx * cx * cz * cz) +
          3.0 * cx * sy * sz * st / Re;
      if (with_pressure) f += -cx * sy * sz * st;
      return f;
    default:
      f = 2.0 * cx * cy * cz * ct - 2.0 * st * st * sz * cz * (sx * sx * cy * cy + cx * cx * sy * sy + 2.0 * cx * cx * cy * cy) +
          6.0 * cx * cy * cz * st / Re;
      if (with_pressure) f += cx * cy * cz * st;
      return f;
  }
}

#ifdef __cplusplus
}
#endif

#endif
