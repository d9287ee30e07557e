/*
 * C-callable harness around the REFERENCE's own hot-path sources — TEST
 * INFRASTRUCTURE ONLY. oracle/Makefile compiles this file together with the
 * reference's src/*.cpp and deps/2Decomp_C/*.cpp (where they lie, read-only)
 * against the single-rank MPI and FFTW stand-ins in oracle/shim/, producing
 * oracle/_ref/libmifref.so. Tests load it through ctypes to pin the CPU
 * restatement (oracle/mif_oracle.c) and to generate the golden fixtures.
 *
 * Field ids: 0..2 velocity u,v,w; 3..5 velocity_buffer; 6..8 velocity_buffer_2;
 * 9 pressure; 10 pressure_buffer (the Poisson solution phi).
 * Call sites mirrored: test/full_test.cpp:60-175 (set-up, step loop, norms),
 * test/pressure_test_hn.cpp:40-70 (stand-alone Poisson solve),
 * test/velocity_test.cpp:75-90 (velocity-only step),
 * src/main.cpp:162-172 and test/full_test.cpp:177-183 (VTK and DAT export).
 */
#include <array>
#include <cstring>
#include <functional>
#include <memory>

#include "Constants.h"
#include "Norms.h"
#include "PressureEquation.h"
#include "PressureGradient.h"
#include "PressureSolverStructures.h"
#include "PressureTensor.h"
#include "StaggeredTensorMacros.h"
#include "Timestep.h"
#include "VTKDatExport.h"
#include "VelocityTensor.h"
#include "manufactured.h"

// include/Timestep.h and include/TimestepVelocity.h share the include guard
// TIMESTEP_VELOCITY_H, so only one of them can be included per translation
// unit; this repeats the declaration of include/TimestepVelocity.h:15-16.
// src/Timestep.cpp:66-81 defines the two projection helpers with external
// linkage but no header declares them; these lines repeat their signatures.
namespace mif {
void timestep_velocity(VelocityTensor &velocity, VelocityTensor &velocity_buffer, VelocityTensor &rhs_buffer,
                       const TimeVectorFunction &exact_velocity, Real t_n);
void update_velocity_pressure_gradient(VelocityTensor &velocity, const StaggeredTensor &pressure, Real delta_time);
void update_pressure(StaggeredTensor &pressure, const StaggeredTensor &pressure_difference);
}

// Globals the reference's generated headers declare (include/Manufactured*.h).
double Reynolds = 1.0;
static int g_forcing_kind = MF_SINCOS;

// The reference's velocity-only step adds forcing_{x,y,z}
// (include/MomentumEquationForcing.h:10-32), generated from
// generators/manufsol_velocity.py. Supplied here from the same formula.
double forcing_x(double t, double x, double y, double z) { return mf_forcing(g_forcing_kind, 0, t, x, y, z, Reynolds, 0); }
double forcing_y(double t, double x, double y, double z) { return mf_forcing(g_forcing_kind, 1, t, x, y, z, Reynolds, 0); }
double forcing_z(double t, double x, double y, double z) { return mf_forcing(g_forcing_kind, 2, t, x, y, z, Reynolds, 0); }

extern "C" {

typedef struct {
  long n_global[3];
  double size[3];
  double origin[3];
  double Re;
  double dt;
  int periodic[3];
  int exact_kind;
} mifref_params;

}  // extern "C"

namespace {

struct RefState {
  int kind;
  double Re;
  std::unique_ptr<mif::Constants> constants;
  std::unique_ptr<mif::PressureSolverStructures> structures;
  std::unique_ptr<mif::VelocityTensor> vel[3];
  std::unique_ptr<mif::StaggeredTensor> pressure;
  std::unique_ptr<mif::StaggeredTensor> pressure_buffer;
  std::unique_ptr<mif::PressureTensor> solver_buffer;
  std::unique_ptr<mif::TimeVectorFunction> exact_velocity;
  std::unique_ptr<mif::TimeVectorFunction> exact_pressure_gradient;

  mif::StaggeredTensor *field(int id) {
    if (id >= 0 && id < 9) return vel[id / 3]->components[id % 3];
    if (id == 9) return pressure.get();
    if (id == 10) return pressure_buffer.get();
    return nullptr;
  }
};

}  // namespace

extern "C" {

void *mifref_create(const mifref_params *p) {
  auto *s = new RefState();
  s->kind = p->exact_kind;
  s->Re = p->Re;
  Reynolds = p->Re;
  g_forcing_kind = p->exact_kind;
  const std::array<bool, 3> periodic{p->periodic[0] != 0, p->periodic[1] != 0, p->periodic[2] != 0};
  // num_time_steps = 1 and final_time = dt give Constants::dt == dt exactly.
  s->constants = std::make_unique<mif::Constants>(
      p->n_global[0], p->n_global[1], p->n_global[2], p->size[0], p->size[1], p->size[2], p->origin[0],
      p->origin[1], p->origin[2], p->Re, p->dt, 1u, 1, 1, 0, periodic);
  s->structures = std::make_unique<mif::PressureSolverStructures>(*s->constants);
  for (int b = 0; b < 3; ++b) s->vel[b] = std::make_unique<mif::VelocityTensor>(*s->constants);
  s->pressure = std::make_unique<mif::StaggeredTensor>(*s->constants, mif::StaggeringDirection::none);
  s->pressure_buffer = std::make_unique<mif::StaggeredTensor>(*s->constants, mif::StaggeringDirection::none);
  s->solver_buffer = std::make_unique<mif::PressureTensor>(*s->structures);
  const int kind = s->kind;
  const double Re = s->Re;
  s->exact_velocity = std::make_unique<mif::TimeVectorFunction>(
      [kind, Re](Real t, Real x, Real y, Real z) { return mf_eval(kind, 0, t, x, y, z, Re); },
      [kind, Re](Real t, Real x, Real y, Real z) { return mf_eval(kind, 1, t, x, y, z, Re); },
      [kind, Re](Real t, Real x, Real y, Real z) { return mf_eval(kind, 2, t, x, y, z, Re); });
  s->exact_pressure_gradient = std::make_unique<mif::TimeVectorFunction>(
      [kind, Re](Real t, Real x, Real y, Real z) { return mf_pressure_gradient(kind, 0, t, x, y, z, Re); },
      [kind, Re](Real t, Real x, Real y, Real z) { return mf_pressure_gradient(kind, 1, t, x, y, z, Re); },
      [kind, Re](Real t, Real x, Real y, Real z) { return mf_pressure_gradient(kind, 2, t, x, y, z, Re); });
  return s;
}

void mifref_destroy(void *h) { delete static_cast<RefState *>(h); }

int mifref_extent(void *h, int id, long out[3]) {
  auto *f = static_cast<RefState *>(h)->field(id);
  if (!f) return -1;
  for (int d = 0; d < 3; ++d) out[d] = (long)f->sizes()[d];
  return 0;
}

int mifref_set(void *h, int id, const double *data) {
  auto *f = static_cast<RefState *>(h)->field(id);
  if (!f) return -1;
  std::memcpy(f->raw_data(), data, sizeof(double) * f->size(f->TOTAL_DATA_COUNT));
  return 0;
}

int mifref_get(void *h, int id, double *data) {
  auto *f = static_cast<RefState *>(h)->field(id);
  if (!f) return -1;
  std::memcpy(data, f->raw_data(), sizeof(double) * f->size(f->TOTAL_DATA_COUNT));
  return 0;
}

// velocity_set(exact(t), include_border) as in test/full_test.cpp:86.
int mifref_set_exact_velocity(void *h, int set, double t, int include_border) {
  auto *s = static_cast<RefState *>(h);
  s->vel[set]->set(s->exact_velocity->set_time(t), include_border != 0);
  return 0;
}

int mifref_set_exact_pressure(void *h, double t) {
  auto *s = static_cast<RefState *>(h);
  const int kind = s->kind;
  const double Re = s->Re;
  s->pressure->set([kind, Re, t](Real x, Real y, Real z) { return mf_eval(kind, 3, t, x, y, z, Re); }, true);
  return 0;
}

// One full projection step, src/Timestep.cpp:151-156.
int mifref_timestep(void *h, double t_n) {
  auto *s = static_cast<RefState *>(h);
  mif::timestep(*s->vel[0], *s->vel[1], *s->vel[2], *s->exact_velocity, t_n, *s->pressure, *s->pressure_buffer,
                *s->solver_buffer);
  return 0;
}

// Same with non-homogeneous Neumann pressure data, src/Timestep.cpp:143-149.
int mifref_timestep_nhn(void *h, double t_n) {
  auto *s = static_cast<RefState *>(h);
  mif::timestep_nhn(*s->vel[0], *s->vel[1], *s->vel[2], *s->exact_velocity, *s->exact_pressure_gradient, t_n,
                    *s->pressure, *s->pressure_buffer, *s->solver_buffer);
  return 0;
}

// Velocity-only step with forcing, src/TimestepVelocity.cpp:60-90
// (set 1 = velocity_buffer, set 2 = rhs_buffer).
int mifref_timestep_velocity(void *h, double t_n) {
  auto *s = static_cast<RefState *>(h);
  mif::timestep_velocity(*s->vel[0], *s->vel[1], *s->vel[2], *s->exact_velocity, t_n);
  return 0;
}

// Stand-alone Poisson solve on velocity set `set`, src/PressureEquation.cpp:266-274.
int mifref_solve_pressure(void *h, int set, double dt) {
  auto *s = static_cast<RefState *>(h);
  mif::solve_pressure_equation_homogeneous_periodic(*s->pressure_buffer, *s->solver_buffer, *s->vel[set], dt);
  return 0;
}

int mifref_solve_pressure_nhn(void *h, int set, double dt, double t_new, double t_old) {
  auto *s = static_cast<RefState *>(h);
  mif::solve_pressure_equation_non_homogeneous_neumann(
      *s->pressure_buffer, *s->solver_buffer, *s->vel[set],
      s->exact_pressure_gradient->get_difference_over_time(t_new, t_old), dt);
  return 0;
}

// Pressure accumulation and gradient correction on velocity set `set`, the
// pair the step runs after each Poisson solve: update_pressure then
// update_velocity_pressure_gradient (src/Timestep.cpp:66-81; both have
// external linkage there, no header declares them).
int mifref_project(void *h, int set, double dt) {
  auto *s = static_cast<RefState *>(h);
  mif::update_pressure(*s->pressure, *s->pressure_buffer);
  mif::update_velocity_pressure_gradient(*s->vel[set], *s->pressure_buffer, dt);
  return 0;
}

// Boundary fill, src/VelocityTensor.cpp:36-233.
int mifref_apply_bc(void *h, int set, double t) {
  auto *s = static_cast<RefState *>(h);
  s->vel[set]->apply_bc(s->exact_velocity->set_time(t));
  return 0;
}

// Mean shift of the pressure, src/PressureEquation.cpp:288-343.
int mifref_adjust_pressure(void *h, double t) {
  auto *s = static_cast<RefState *>(h);
  const int kind = s->kind;
  const double Re = s->Re;
  mif::adjust_pressure(*s->pressure, [kind, Re, t](Real x, Real y, Real z) { return mf_eval(kind, 3, t, x, y, z, Re); });
  return 0;
}

// The nine numbers of test/full_test.cpp:150-175: L1, L2, Linf of velocity,
// pressure and pressure gradient against the exact fields at time t
// (no pressure adjustment here; call mifref_adjust_pressure first if wanted).
int mifref_error_norms(void *h, double t, double out[9]) {
  auto *s = static_cast<RefState *>(h);
  const mif::Constants &constants = *s->constants;
  mif::VelocityTensor &velocity = *s->vel[0];
  mif::StaggeredTensor &pressure = *s->pressure;
  const int kind = s->kind;
  const double Re = s->Re;
  std::function<Real(Real, Real, Real, Real)> p_exact = [kind, Re](Real tt, Real x, Real y, Real z) {
    return mf_eval(kind, 3, tt, x, y, z, Re);
  };
  mif::VelocityTensor pressure_gradient(constants);
  VELOCITY_TENSOR_SET_FOR_ALL_POINTS(pressure_gradient, mif::pressure_gradient_u, mif::pressure_gradient_v,
                                     mif::pressure_gradient_w, false, pressure, i, j, k)
  pressure_gradient.apply_bc(s->exact_pressure_gradient->set_time(t));
  out[0] = mif::ErrorL1Norm(velocity, *s->exact_velocity, t);
  out[1] = mif::ErrorL2Norm(velocity, *s->exact_velocity, t);
  out[2] = mif::ErrorLInfNorm(velocity, *s->exact_velocity, t);
  out[3] = mif::ErrorL1Norm(pressure, p_exact, t);
  out[4] = mif::ErrorL2Norm(pressure, p_exact, t);
  out[5] = mif::ErrorLInfNorm(pressure, p_exact, t);
  out[6] = mif::ErrorL1Norm(pressure_gradient, *s->exact_pressure_gradient, t);
  out[7] = mif::ErrorL2Norm(pressure_gradient, *s->exact_pressure_gradient, t);
  out[8] = mif::ErrorLInfNorm(pressure_gradient, *s->exact_pressure_gradient, t);
  return 0;
}

// The reference's exporters on velocity set 0 and the pressure
// (include/VTKDatExport.h:10-29).
int mifref_write_vtk(void *h, const char *filename) {
  auto *s = static_cast<RefState *>(h);
  mif::writeVTK(filename, *s->vel[0], *s->pressure);
  return 0;
}
int mifref_write_dat(void *h, const char *filename, int direction, double x, double y, double z) {
  auto *s = static_cast<RefState *>(h);
  mif::writeDat(filename, *s->vel[0], *s->pressure, direction, x, y, z);
  return 0;
}
int mifref_write_vtk_full_mesh(void *h, const char *filename) {
  auto *s = static_cast<RefState *>(h);
  mif::writeVTKFullMesh(filename, *s->vel[0], *s->pressure);
  return 0;
}

}  // extern "C"
