// Shared definitions of the mifgpu CUDA library (sm_103a).
//
// Device layout. Every field of a context (the nine velocity components of
// the three velocity sets, the pressure and the Poisson solution phi) lives in
// one common padded box of PX x PY x PZ elements, x fastest:
//     idx(i, j, k) = i + PX * (j + PY * k)
// with PX >= the largest x extent over all fields (rounded up to 8 elements so
// rows start 32-byte aligned), PY and PZ the largest y and z extents. A field
// only uses its own extents (the reference's, src/StaggeredTensor.cpp:5-9);
// the padding is never read by a stencil. Sharing one index space means every
// stencil neighbour is the same offset (+-1, +-PX, +-PX*PY) for all fields, so
// the fused kernels need a single address per point.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace mifgpu {

constexpr int kFieldsPerSet = 3;
constexpr int kNumFields = 11;  // 9 velocity components, p, phi
constexpr int kP = 9;
constexpr int kPhi = 10;

// Grid constants of src/Constants.cpp:58-120 for one rank, plus the device
// pitches. Passed by value to every kernel.
struct Geometry {
  int n_global[3];
  int periodic[3];
  int E[3];       // Nx, Ny, Nz (pressure / unstaggered extents)
  int Es[3];      // Nx_staggered, Ny_staggered, Nz_staggered
  int base[3];    // base_i, base_j, base_k
  int np[3];      // Poisson points per axis (src/PressureSolverStructures.cpp:15-17)
  int own_lo[3];  // first owner index per axis (1 if periodic, else 0)
  long PX, PY, PZ;
  double origin[3];
  double h[3], oh[3], o2h[3], o8h[3], oh2Re[3], h_2[3];
  double Re, dt;

  __host__ __device__ long idx(long i, long j, long k) const { return i + PX * (j + PY * k); }
  __host__ __device__ long sy() const { return PX; }
  __host__ __device__ long sz() const { return PX * PY; }
  // Extent of component c (0 u, 1 v, 2 w) along axis d.
  __host__ __device__ int ext(int c, int d) const { return c == d ? Es[d] : E[d]; }
  __host__ __device__ double node(int d, long i) const { return origin[d] + h[d] * (double)(base[d] + i); }
  __host__ __device__ double face(int d, long i) const { return node(d, i) - h_2[d]; }
};

// Stencil coefficients in the working precision T.
template <typename T>
struct Coeffs {
  T o2h[3], o8h[3], oh2Re[3], oh[3];
};

// Compensated float state (MIFGPU_MIXED_COMPENSATED): each velocity
// component of the state carries a bfloat16 residual, so the value is
// hi + lo with hi the float field and lo what the float update rounded away
// (about 32 significant bits in all). One residual triple serves every
// velocity set: each kernel that writes a state reads the residual of its
// input state at the same point and overwrites it with the residual of its
// output state. c[0] == nullptr: no compensation (FP64, MIXED).
struct Residual {
  __nv_bfloat16 *c[3] = {nullptr, nullptr, nullptr};
  __host__ __device__ bool on() const { return c[0] != nullptr; }
};

// hi + (lo + inc) as an error-free float sum (Knuth's TwoSum on hi and
// t = lo + inc): returns the new hi and stores the rounding error, rounded to
// bfloat16, as the new residual. Exact for any magnitudes; the only losses are
// the float rounding of t (2^-24 |t|, with |t| about ulp(hi) + |inc|) and the
// bfloat16 rounding of the residual (2^-9 of half an ulp of hi).
__device__ __forceinline__ float comp_add(float hi, float lo, float inc, __nv_bfloat16 *lo_out) {
  const float t = __fadd_rn(lo, inc);
  const float s = __fadd_rn(hi, t);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(t, bb));
  *lo_out = __float2bfloat16_rn(e);
  return s;
}

// A double value split into its float part and the bfloat16 residual.
__device__ __forceinline__ float comp_split(double v, __nv_bfloat16 *lo_out) {
  const float hi = (float)v;
  *lo_out = __float2bfloat16_rn((float)(v - (double)hi));
  return hi;
}

template <typename T>
struct Vec2;
template <>
struct Vec2<float> {
  using type = float2;
};
template <>
struct Vec2<double> {
  using type = double2;
};

}  // namespace mifgpu
