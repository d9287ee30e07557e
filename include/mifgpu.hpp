// C++ host mirror of the reference's time-step interface over the mifgpu C ABI.
//
// The reference's entry points take its own tensor classes
// (include/Timestep.h:16-27, include/TimestepVelocity.h:15-16,
// include/PressureEquation.h:10-25). This header keeps their names and
// argument meaning but works on anything that exposes a contiguous buffer in
// the reference layout (x fastest, the reference's extents): raw pointers, or
// the reference's StaggeredTensor through raw_data(). Errors throw
// mifgpu::Error carrying the library message; the reference asserts instead
// (compiled out under NDEBUG), so a caller that wants its behaviour can catch
// and abort.
#ifndef MIFGPU_HPP
#define MIFGPU_HPP

#include <array>
#include <stdexcept>
#include <string>

#include "mifgpu.h"

namespace mifgpu {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &what) : std::runtime_error(what), code(c) {}
};

// The reference's field ids of include/mifgpu.h.
enum Field { U = 0, V = 1, W = 2, U1 = 3, V1 = 4, W1 = 5, U2 = 6, V2 = 7, W2 = 8, P = 9, PHI = 10 };

// Grid and physics of src/Constants.cpp:58-120 for one rank.
struct Constants {
  std::array<long, 3> n_global;            // include/Constants.h:14-16 convention
  std::array<double, 3> size{1.0, 1.0, 1.0};
  std::array<double, 3> origin{0.0, 0.0, 0.0};
  double Re = 1000.0;
  double dt = 1e-4;
  std::array<bool, 3> periodic_bc{false, false, false};
  int precision = MIFGPU_FP64;
  int boundary_kind = MIFGPU_FIELD_ZERO;
  int forcing = MIFGPU_FORCING_NONE;
  double forcing_amplitude = 0.0;
};

// Owns the device state: what the reference holds in Constants,
// PressureSolverStructures and the six tensors of src/main.cpp:127-141.
class Solver {
 public:
  explicit Solver(const Constants &c) {
    mifgpu_params p{};
    for (int d = 0; d < 3; ++d) {
      p.n_global[d] = c.n_global[d];
      p.size[d] = c.size[d];
      p.origin[d] = c.origin[d];
      p.periodic[d] = c.periodic_bc[d] ? 1 : 0;
    }
    p.Re = c.Re;
    p.dt = c.dt;
    p.precision = c.precision;
    p.boundary_kind = c.boundary_kind;
    p.forcing = c.forcing;
    p.forcing_amplitude = c.forcing_amplitude;
    const int rc = mifgpu_create(&p, &ctx_);
    if (rc != MIFGPU_OK) {
      const std::string msg = ctx_ ? mifgpu_last_error(ctx_) : "invalid parameters";
      if (ctx_) mifgpu_destroy(ctx_);
      ctx_ = nullptr;
      throw Error(rc, "mifgpu_create: " + msg);
    }
  }
  ~Solver() {
    if (ctx_) mifgpu_destroy(ctx_);
  }
  Solver(const Solver &) = delete;
  Solver &operator=(const Solver &) = delete;

  std::array<long, 3> extent(Field f) const {
    std::array<long, 3> e{};
    check(mifgpu_field_extent(ctx_, f, e.data()), "field_extent");
    return e;
  }
  void upload(Field f, const double *host) { check(mifgpu_upload(ctx_, f, host), "upload"); }
  void download(Field f, double *host) { check(mifgpu_download(ctx_, f, host), "download"); }

  // mif::timestep (src/Timestep.cpp:151-156) on host buffers of velocity and
  // pressure: the three velocity buffers and the pressure buffers of the
  // reference's signature live on the device.
  void timestep(double *u, double *v, double *w, double t_n, double *pressure) {
    check(mifgpu_timestep_host(ctx_, t_n, u, v, w, pressure), "timestep");
  }
  // Device-resident forms.
  void timestep(double t_n) { check(mifgpu_timestep(ctx_, t_n), "timestep"); }
  void run(double t0, int nsteps) { check(mifgpu_run(ctx_, t0, nsteps), "run"); }
  void timestep_nhn(double t_n) { check(mifgpu_timestep_nhn(ctx_, t_n), "timestep_nhn"); }
  void timestep_velocity(double t_n) { check(mifgpu_timestep_velocity(ctx_, t_n), "timestep_velocity"); }
  void run_velocity(double t0, int nsteps) { check(mifgpu_run_velocity(ctx_, t0, nsteps), "run_velocity"); }
  void solve_pressure_equation_homogeneous_periodic(int velocity_set, double dt) {
    check(mifgpu_solve_pressure(ctx_, velocity_set, dt), "solve_pressure");
  }
  void apply_bc(int velocity_set, double t) { check(mifgpu_apply_bc(ctx_, velocity_set, t), "apply_bc"); }

  // Caller boundary data (boundary_kind MIFGPU_FIELD_CALLER): the Dirichlet
  // face planes of u, v, w for time slot `slot` (0: apply_bc; 1..3: the
  // stages of the next step), and the normal pressure-gradient faces of the
  // non-homogeneous Neumann step.
  void set_boundary_values(int slot, const double *u, const double *v, const double *w) {
    check(mifgpu_set_boundary_values(ctx_, slot, u, v, w), "set_boundary_values");
  }
  void set_pressure_gradient_faces(int slot, const std::array<const double *, 6> &faces) {
    check(mifgpu_set_pressure_gradient_faces(ctx_, slot, faces.data()), "set_pressure_gradient_faces");
  }
  // solve_pressure_equation_non_homogeneous_neumann (include/PressureEquation.h:15-19)
  // with the caller's normal pressure-gradient faces.
  void solve_pressure_equation_non_homogeneous_neumann(int velocity_set, double dt,
                                                       const std::array<const double *, 6> &faces) {
    check(mifgpu_solve_pressure_nhn(ctx_, velocity_set, dt, faces.data()), "solve_pressure_nhn");
  }
  void adjust_pressure(double t) { check(mifgpu_adjust_pressure(ctx_, t), "adjust_pressure"); }
  std::array<double, 9> error_norms(double t) {
    std::array<double, 9> out{};
    check(mifgpu_error_norms(ctx_, t, out.data()), "error_norms");
    return out;
  }
  void set_exact_velocity(int set, double t) { check(mifgpu_set_exact_velocity(ctx_, set, t), "set_exact_velocity"); }
  void set_exact_pressure(double t) { check(mifgpu_set_exact_pressure(ctx_, t), "set_exact_pressure"); }

  // The two halves of the step around the Poisson solve:
  // calculate_velocity_divergence (include/VelocityDivergence.h:9-20) into
  // the pressure buffer, and update_pressure + update_velocity_pressure_gradient
  // (src/Timestep.cpp:66-81).
  void calculate_velocity_divergence(int velocity_set, double dt) {
    check(mifgpu_divergence(ctx_, velocity_set, dt), "divergence");
  }
  void update_pressure_and_velocity(int velocity_set, double dt) {
    check(mifgpu_project(ctx_, velocity_set, dt), "project");
  }

  // writeVTK, writeDat, writeVTKFullMesh (include/VTKDatExport.h:10-29) from
  // the device-resident fields; the same bytes as the reference's writers.
  void writeVTK(const std::string &filename) { check(mifgpu_write_vtk(ctx_, filename.c_str()), "write_vtk"); }
  void writeDat(const std::string &filename, int direction, double x, double y, double z) {
    check(mifgpu_write_dat(ctx_, filename.c_str(), direction, x, y, z), "write_dat");
  }
  void writeVTKFullMesh(const std::string &filename) {
    check(mifgpu_write_vtk_full_mesh(ctx_, filename.c_str()), "write_vtk_full_mesh");
  }

  // Stream control: `stream` is a cudaStream_t (nullptr: the context's own).
  void set_stream(void *stream) { check(mifgpu_set_stream(ctx_, stream), "set_stream"); }
  void synchronize() { check(mifgpu_synchronize(ctx_), "synchronize"); }

  // Reverse mode (no counterpart in the reference): see include/mifgpu.h.
  // Each returns d loss / d forcing_amplitude (0 unless the forcing is
  // MIFGPU_FORCING_TAYLOR_GREEN); ms, when non-null, receives the
  // milliseconds of the forward pass, the segment recomputes and the reverse
  // sweeps.
  double gradient_ke(double t0, int nsteps, int checkpoint_every, const std::array<double, 6> &box, double *loss,
                     std::array<double, 3> *ms = nullptr) {
    double dalpha = 0.0;
    std::array<double, 3> t{};
    check(mifgpu_gradient_ke(ctx_, t0, nsteps, checkpoint_every, box.data(), loss, &dalpha, t.data()),
          "gradient_ke");
    if (ms) *ms = t;
    return dalpha;
  }
  double backward(double t0, int nsteps, int checkpoint_every, const double *seed_u, const double *seed_v,
                  const double *seed_w, const double *seed_p, std::array<double, 3> *ms = nullptr) {
    double dalpha = 0.0;
    std::array<double, 3> t{};
    check(mifgpu_backward(ctx_, t0, nsteps, checkpoint_every, seed_u, seed_v, seed_w, seed_p, &dalpha, t.data()),
          "backward");
    if (ms) *ms = t;
    return dalpha;
  }
  void download_adjoint(Field f, double *host) { check(mifgpu_download_adjoint(ctx_, f, host), "download_adjoint"); }
  void set_forcing_amplitude(double alpha) {
    check(mifgpu_set_forcing_amplitude(ctx_, alpha), "set_forcing_amplitude");
  }

  // Velocity error norms (L1, L2, Linf) that allocate nothing.
  std::array<double, 3> velocity_error_norms_noalloc(double t) {
    std::array<double, 3> out{};
    check(mifgpu_velocity_error_norms_noalloc(ctx_, t, out.data()), "velocity_error_norms_noalloc");
    return out;
  }

  // Instrumentation (no counterpart in the reference).
  std::array<double, MIFGPU_PROF_CLASSES> profile_step(double t_n, int reps) {
    std::array<double, MIFGPU_PROF_CLASSES> ms{};
    check(mifgpu_profile_step(ctx_, t_n, reps, ms.data()), "profile_step");
    return ms;
  }
  long long launch_count() const {
    long long n = 0;
    check(mifgpu_launch_count(ctx_, &n), "launch_count");
    return n;
  }
  size_t device_bytes() const {
    size_t n = 0;
    check(mifgpu_device_bytes(ctx_, &n), "device_bytes");
    return n;
  }
  // The current device's FP64 FMA rate in TFLOP/s; needs no context.
  static double probe_fp64_fma() {
    double tflops = 0.0;
    const int rc = mifgpu_probe_fp64_fma(&tflops);
    if (rc != MIFGPU_OK) throw Error(rc, "probe_fp64_fma failed");
    return tflops;
  }

  mifgpu_ctx *handle() { return ctx_; }

 private:
  void check(int rc, const char *what) const {
    if (rc != MIFGPU_OK) throw Error(rc, std::string(what) + ": " + mifgpu_last_error(ctx_));
  }
  mifgpu_ctx *ctx_ = nullptr;
};

}  // namespace mifgpu

#endif  // MIFGPU_HPP
