// Analytic velocity / pressure families, evaluated on the device.
//
// The reference passes boundary data and forcing as host std::function
// objects (include/VectorFunction.h:33-53); a GPU step cannot call back to the
// host, so the families the reference's tests and benchmarks use are compiled
// in (enum mifgpu_field_kind):
//   SINCOS: the velocity of generators/manufsol_velocity.py:55-57 with the
//           pressure p = cos x cos y sin z sin t;
//   ETHIER: the exact Navier-Stokes solution of generators/manufsol.py:35-72.
// TE is the evaluation precision: double in FP64 mode, float in mixed mode.
#pragma once

#include "common.cuh"

namespace mifgpu {

enum { kFieldZero = 0, kFieldSincos = 1, kFieldEthier = 2, kFieldCaller = 3 };  // kFieldCaller: no analytic field

template <typename TE>
__device__ __forceinline__ TE an_sin(TE x);
template <>
__device__ __forceinline__ double an_sin(double x) { return sin(x); }
template <>
__device__ __forceinline__ float an_sin(float x) { return sinf(x); }
template <typename TE>
__device__ __forceinline__ TE an_cos(TE x);
template <>
__device__ __forceinline__ double an_cos(double x) { return cos(x); }
template <>
__device__ __forceinline__ float an_cos(float x) { return cosf(x); }
template <typename TE>
__device__ __forceinline__ TE an_exp(TE x);
template <>
__device__ __forceinline__ double an_exp(double x) { return exp(x); }
template <>
__device__ __forceinline__ float an_exp(float x) { return expf(x); }

// comp 0..2 velocity, 3 pressure.
template <typename TE>
__device__ TE analytic_value(int kind, int comp, TE t, TE x, TE y, TE z, TE Re) {
  if (kind == kFieldSincos) {
    const TE st = an_sin(t);
    switch (comp) {
      case 0: return an_sin(x) * an_cos(y) * an_sin(z) * st;
      case 1: return an_cos(x) * an_sin(y) * an_sin(z) * st;
      case 2: return TE(2) * an_cos(x) * an_cos(y) * an_cos(z) * st;
      default: return an_cos(x) * an_cos(y) * an_sin(z) * st;
    }
  }
  if (kind == kFieldEthier) {
    const TE a = TE(0.78539816339744830962), d = TE(1.57079632679489661923);
    const TE decay = an_exp(-d * d * t / Re);
    switch (comp) {
      case 0: return -a * (an_exp(a * x) * an_sin(a * y + d * z) + an_exp(a * z) * an_cos(a * x + d * y)) * decay;
      case 1: return -a * (an_exp(a * y) * an_sin(a * z + d * x) + an_exp(a * x) * an_cos(a * y + d * z)) * decay;
      case 2: return -a * (an_exp(a * z) * an_sin(a * x + d * y) + an_exp(a * y) * an_cos(a * z + d * x)) * decay;
      default: {
        const TE A = a * x + d * y, B = a * y + d * z, C = a * z + d * x;
        return -a * a / TE(2) *
               (an_exp(TE(2) * a * x) + an_exp(TE(2) * a * y) + an_exp(TE(2) * a * z) +
                TE(2) * an_sin(A) * an_cos(C) * an_exp(a * (y + z)) + TE(2) * an_sin(B) * an_cos(A) * an_exp(a * (z + x)) +
                TE(2) * an_sin(C) * an_cos(B) * an_exp(a * (x + y))) *
               decay * decay;
      }
    }
  }
  return TE(0);
}

// d p / d x_comp of the family's pressure.
template <typename TE>
__device__ TE analytic_pressure_gradient(int kind, int comp, TE t, TE x, TE y, TE z, TE Re) {
  if (kind == kFieldSincos) {
    const TE st = an_sin(t);
    switch (comp) {
      case 0: return -an_sin(x) * an_cos(y) * an_sin(z) * st;
      case 1: return -an_cos(x) * an_sin(y) * an_sin(z) * st;
      default: return an_cos(x) * an_cos(y) * an_cos(z) * st;
    }
  }
  if (kind == kFieldEthier) {
    const TE a = TE(0.78539816339744830962), d = TE(1.57079632679489661923);
    const TE decay2 = an_exp(TE(-2) * d * d * t / Re);
    TE X = x, Y = y, Z = z;
    if (comp == 1) X = y, Y = z, Z = x;
    if (comp == 2) X = z, Y = x, Z = y;
    const TE A = a * X + d * Y, B = a * Y + d * Z, C = a * Z + d * X;
    const TE s = TE(2) * a * an_exp(TE(2) * a * X) +
                 TE(2) * an_exp(a * (Y + Z)) * (a * an_cos(A) * an_cos(C) - d * an_sin(A) * an_sin(C)) +
                 TE(2) * a * an_sin(B) * an_exp(a * (Z + X)) * (an_cos(A) - an_sin(A)) +
                 TE(2) * an_cos(B) * an_exp(a * (X + Y)) * (d * an_cos(C) + a * an_sin(C));
    return -a * a / TE(2) * s * decay2;
  }
  return TE(0);
}

// fn 0: velocity family, 1: pressure-gradient family.
template <typename TE>
__device__ __forceinline__ TE analytic_vector(int fn, int kind, int comp, TE t, TE x, TE y, TE z, TE Re) {
  return fn == 0 ? analytic_value<TE>(kind, comp, t, x, y, z, Re)
                 : analytic_pressure_gradient<TE>(kind, comp, t, x, y, z, Re);
}

}  // namespace mifgpu
