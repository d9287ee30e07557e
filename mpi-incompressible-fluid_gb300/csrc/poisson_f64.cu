// double instantiation of the spectral Poisson solver (poisson_impl.cuh).
#include "poisson_impl.cuh"

namespace mifgpu {
template struct AxisPlan<double>;
template struct PoissonSolver<double>;
}  // namespace mifgpu
