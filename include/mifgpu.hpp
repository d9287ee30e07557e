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
  void solve_pressure_equation_homogeneous_periodic(int velocity_set, double dt) {
    check(mifgpu_solve_pressure(ctx_, velocity_set, dt), "solve_pressure");
  }
  void apply_bc(int velocity_set, double t) { check(mifgpu_apply_bc(ctx_, velocity_set, t), "apply_bc"); }
  void adjust_pressure(double t) { check(mifgpu_adjust_pressure(ctx_, t), "adjust_pressure"); }
  std::array<double, 9> error_norms(double t) {
    std::array<double, 9> out{};
    check(mifgpu_error_norms(ctx_, t, out.data()), "error_norms");
    return out;
  }
  void set_exact_velocity(int set, double t) { check(mifgpu_set_exact_velocity(ctx_, set, t), "set_exact_velocity"); }
  void set_exact_pressure(double t) { check(mifgpu_set_exact_pressure(ctx_, t), "set_exact_pressure"); }
  mifgpu_ctx *handle() { return ctx_; }

 private:
  void check(int rc, const char *what) const {
    if (rc != MIFGPU_OK) throw Error(rc, std::string(what) + ": " + mifgpu_last_error(ctx_));
  }
  mifgpu_ctx *ctx_ = nullptr;
};

}  // namespace mifgpu

#endif  // MIFGPU_HPP
