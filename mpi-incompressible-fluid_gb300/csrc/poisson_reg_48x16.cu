// Register-path line kernels of FFT shape 48 x 16 (float), compiled on their own.
#define MIFGPU_REG_TU
#include "poisson_impl.cuh"

namespace mifgpu {
template const void *reg_kernel_ptr<float, 48, 16>(int, int);
}  // namespace mifgpu
