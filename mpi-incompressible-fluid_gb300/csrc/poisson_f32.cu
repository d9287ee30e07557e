// float instantiation of the spectral Poisson solver (poisson_impl.cuh).
#include "poisson_impl.cuh"

namespace mifgpu {
template struct AxisPlan<float>;
template struct PoissonSolver<float>;
}  // namespace mifgpu
