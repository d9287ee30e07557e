// Velocity error norms that allocate nothing (norms_noalloc.cu).
#pragma once

#include <string>

#include "common.cuh"

namespace mifgpu {

// Interior z planes the static scratch has room for: 3 partial sums per plane
// plus the 3 results, (4000 + 1) * 3 doubles = 96 KB.
constexpr int kNoAllocMaxPlanes = 4000;

// Device address of the scratch on the current device, looked up with
// cudaGetSymbolAddress once per device and context and cached. Returns 0, or
// -2 with `err` set.
int noalloc_scratch(double **out, std::string &err);

// Two-pass reduction of src/Norms.cpp:11-47 over velocity set (u, v, w):
// one block per interior z plane writes that plane's (sum |e|, sum e^2,
// max |e|) to scratch[3 k], then one block adds the planes in index order and
// writes the three totals to scratch[3 kNoAllocMaxPlanes]. Every scratch
// element read is written earlier in the same call, so nothing has to start
// at zero. Needs E[2] - 2 <= kNoAllocMaxPlanes (the caller checks). With `res`
// on, the velocity is hi + residual (the compensated state).
template <typename T>
void launch_velocity_errors_noalloc(const Geometry &g, const T *u, const T *v, const T *w, int field_kind, double t,
                                    double *scratch, cudaStream_t s, long long *launches, const Residual &res);

}  // namespace mifgpu
