// src/Timestep.cpp of the reference's single-GPU build: compile with
// -DMIF_GB300 and link -L<repo>/mpi-incompressible-fluid_gb300 -lmifgpu.
// It replaces the two functions the file defines, mif::timestep and
// mif::timestep_nhn (include/Timestep.h:16-27), for one rank; the
// reference's own file stays whole under #else. The caller's exact_velocity
// and exact_pressure_gradient functions are honoured: the reference's own
// apply_bc evaluates the first at each stage time into a buffer the GPU step
// does not use (velocity_buffer), and the second is sampled at the boundary
// nodes, as apply_non_homogeneous_neumann samples it; the library takes both
// as per-stage data (boundary_kind MIFGPU_FIELD_CALLER).
#ifdef MIF_GB300
#include <array>
#include <cassert>
#include <vector>

#include "Timestep.h"
#include "mifgpu.h"

namespace mif {
namespace {

// One GPU, one solver per process, created on the first step.
mifgpu_ctx *gpu_context(const Constants &c) {
  static mifgpu_ctx *ctx = nullptr;
  if (!ctx) {
    mifgpu_params p{};
    p.n_global[0] = (long)c.Nx_global;
    p.n_global[1] = (long)c.Ny_global;
    p.n_global[2] = (long)c.Nz_global;
    p.size[0] = c.x_size;
    p.size[1] = c.y_size_global;
    p.size[2] = c.z_size_global;
    p.origin[0] = c.min_x_global;
    p.origin[1] = c.min_y_global;
    p.origin[2] = c.min_z_global;
    p.Re = c.Re;
    p.dt = c.dt;
    for (int d = 0; d < 3; ++d) p.periodic[d] = c.periodic_bc[d];
    p.precision = MIFGPU_FP64;
    p.boundary_kind = MIFGPU_FIELD_CALLER;  // the caller's functions, fed per stage below
    p.forcing = MIFGPU_FORCING_NONE;        // mif::timestep has no forcing
    if (mifgpu_create(&p, &ctx) != MIFGPU_OK) MPI_Abort(MPI_COMM_WORLD, 1);
  }
  return ctx;
}

double *raw(StaggeredTensor &t) { return static_cast<double *>(t.raw_data()); }

// The stage times of FULL_TIMESTEP (src/Timestep.cpp:97-104).
std::array<Real, 3> stage_times(const Constants &c, Real t_n) {
  const Real dt_1 = 64.0 / 120.0 * c.dt;
  const Real time_1 = t_n + dt_1;
  const Real dt_2 = 16.0 / 120.0 * c.dt;
  const Real time_2 = time_1 + dt_2;
  return {time_1, time_2, t_n + c.dt};
}

// The Dirichlet values of each stage (src/Timestep.cpp:110,120,130): the
// reference's apply_bc writes them into `scratch`, the library copies its
// face planes.
int feed_boundary(mifgpu_ctx *ctx, VelocityTensor &scratch, const TimeVectorFunction &exact_velocity,
                  const std::array<Real, 3> &times) {
  for (int k = 0; k < 3; ++k) {
    scratch.apply_bc(exact_velocity.set_time(times[k]));
    const int rc = mifgpu_set_boundary_values(ctx, 1 + k, raw(scratch.u), raw(scratch.v), raw(scratch.w));
    if (rc != MIFGPU_OK) return rc;
  }
  return MIFGPU_OK;
}

// The Neumann data of each stage (src/Timestep.cpp:85-90): the normal
// component of get_difference_over_time(t_k, t_{k-1}) at the pressure nodes
// of the six faces, where apply_non_homogeneous_neumann
// (src/PressureEquation.cpp:10-56) evaluates it.
int feed_gradient(mifgpu_ctx *ctx, const StaggeredTensor &p, const TimeVectorFunction &exact_pressure_gradient,
                  Real t_n, const std::array<Real, 3> &times) {
  const std::array<size_t, 3> n = p.sizes();
  const Real prev[3] = {t_n, times[0], times[1]};
  std::vector<double> face[6];
  for (int f = 0; f < 6; ++f) face[f].resize(f < 2 ? n[1] * n[2] : (f < 4 ? n[0] * n[2] : n[0] * n[1]));
  for (int k = 0; k < 3; ++k) {
    const VectorFunction g = exact_pressure_gradient.get_difference_over_time(times[k], prev[k]);
    for (size_t c = 0; c < n[2]; ++c)
      for (size_t b = 0; b < n[1]; ++b) {
        face[0][b + n[1] * c] = p.evaluate_function_at_index(0, b, c, g.f_u);
        face[1][b + n[1] * c] = p.evaluate_function_at_index(n[0] - 1, b, c, g.f_u);
      }
    for (size_t c = 0; c < n[2]; ++c)
      for (size_t a = 0; a < n[0]; ++a) {
        face[2][a + n[0] * c] = p.evaluate_function_at_index(a, 0, c, g.f_v);
        face[3][a + n[0] * c] = p.evaluate_function_at_index(a, n[1] - 1, c, g.f_v);
      }
    for (size_t b = 0; b < n[1]; ++b)
      for (size_t a = 0; a < n[0]; ++a) {
        face[4][a + n[0] * b] = p.evaluate_function_at_index(a, b, 0, g.f_w);
        face[5][a + n[0] * b] = p.evaluate_function_at_index(a, b, n[2] - 1, g.f_w);
      }
    const double *faces[6] = {face[0].data(), face[1].data(), face[2].data(),
                              face[3].data(), face[4].data(), face[5].data()};
    const int rc = mifgpu_set_pressure_gradient_faces(ctx, 1 + k, faces);
    if (rc != MIFGPU_OK) return rc;
  }
  return MIFGPU_OK;
}

}  // namespace

void timestep(VelocityTensor &velocity, VelocityTensor &velocity_buffer, VelocityTensor &,
              const TimeVectorFunction &exact_velocity, Real t_n, StaggeredTensor &pressure, StaggeredTensor &,
              PressureTensor &) {
  assert(velocity.constants.P == 1);
  mifgpu_ctx *ctx = gpu_context(velocity.constants);
  int rc = feed_boundary(ctx, velocity_buffer, exact_velocity, stage_times(velocity.constants, t_n));
  if (rc == MIFGPU_OK)
    rc = mifgpu_timestep_host(ctx, t_n, raw(velocity.u), raw(velocity.v), raw(velocity.w), raw(pressure));
  if (rc != MIFGPU_OK) MPI_Abort(MPI_COMM_WORLD, rc);
}

void timestep_nhn(VelocityTensor &velocity, VelocityTensor &velocity_buffer, VelocityTensor &,
                  const TimeVectorFunction &exact_velocity, const TimeVectorFunction &exact_pressure_gradient,
                  Real t_n, StaggeredTensor &pressure, StaggeredTensor &, PressureTensor &) {
  assert(velocity.constants.P == 1);
  mifgpu_ctx *ctx = gpu_context(velocity.constants);
  const std::array<Real, 3> times = stage_times(velocity.constants, t_n);
  int rc = feed_boundary(ctx, velocity_buffer, exact_velocity, times);
  if (rc == MIFGPU_OK) rc = feed_gradient(ctx, pressure, exact_pressure_gradient, t_n, times);
  double *host[4] = {raw(velocity.u), raw(velocity.v), raw(velocity.w), raw(pressure)};
  const int field[4] = {0, 1, 2, 9};  // velocity.{u,v,w}, pressure
  for (int q = 0; q < 4 && rc == MIFGPU_OK; ++q) rc = mifgpu_upload(ctx, field[q], host[q]);
  if (rc == MIFGPU_OK) rc = mifgpu_timestep_nhn(ctx, t_n);
  for (int q = 0; q < 4 && rc == MIFGPU_OK; ++q) rc = mifgpu_download(ctx, field[q], host[q]);
  if (rc != MIFGPU_OK) MPI_Abort(MPI_COMM_WORLD, rc);
}

}  // namespace mif
#else
// ... the reference's own src/Timestep.cpp, unchanged ...
#endif
