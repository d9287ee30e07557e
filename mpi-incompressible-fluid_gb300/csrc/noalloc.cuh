// Velocity error norms that allocate nothing (norms_noalloc.cu).
#pragma once

#include <string>

#include "common.cuh"

namespace mifgpu {

// Partial-sum slots of the static scratch: 3 partial sums per slot plus the
// 3 results, (4000 + 1) * 3 doubles = 96 KB. Each interior z plane takes at
// least one slot, so this is also the largest number of interior planes.
constexpr int kNoAllocMaxPlanes = 4000;

// Device address of the scratch on the current device, looked up with
// cudaGetSymbolAddress once per device and context and cached. Returns 0, or
// -2 with `err` set.
int noalloc_scratch(double **out, std::string &err);

// Two-pass reduction of src/Norms.cpp:11-47 over velocity set (u, v, w):
// each interior z plane is split into the same number of chunks (as many as
// the slots allow, each of at least 1024 points, so that flat grids fill the
// GPU too); one block per chunk writes its (sum |e|, sum e^2, max |e|) to its
// own slot, then one block adds the slots in index order and writes the three
// totals to scratch[3 kNoAllocMaxPlanes]. The split depends on the grid only,
// so the result is the same on every call. Every scratch
// element read is written earlier in the same call, so nothing has to start
// at zero. Needs E[2] - 2 <= kNoAllocMaxPlanes (the caller checks). With `res`
// on, the velocity is hi + residual (the compensated state).
template <typename T>
void launch_velocity_errors_noalloc(const Geometry &g, const T *u, const T *v, const T *w, int field_kind, double t,
                                    double *scratch, cudaStream_t s, long long *launches, const Residual &res);

}  // namespace mifgpu
