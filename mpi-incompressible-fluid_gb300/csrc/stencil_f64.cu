// double instantiation of the point-wise kernels (stencil_impl.cuh).
#include "stencil_impl.cuh"

namespace mifgpu {
MIFGPU_INSTANTIATE(double)
}  // namespace mifgpu
