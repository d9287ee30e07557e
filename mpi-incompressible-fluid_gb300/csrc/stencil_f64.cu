// double instantiation of the point-wise kernels (stencil_impl.cuh), and the
// precision-independent face-table helpers.
#define MIFGPU_STENCIL_SHARED
#include "stencil_impl.cuh"

namespace mifgpu {
MIFGPU_INSTANTIATE(double)
}  // namespace mifgpu
