/*
 * mifgpu — one GB300 (sm_103a) time step of the staggered-grid incompressible
 * Navier-Stokes solver of FattiMei/mpi-incompressible-fluid, behind a C ABI.
 *
 * The library owns device memory; the caller owns host memory. Host arrays are
 * in the reference's own layout: one StaggeredTensor per field, x fastest,
 * index i + Ex*(j + Ey*k) (include/Tensor.h:137-140,237), with the reference's
 * extents per staggering (src/StaggeredTensor.cpp:5-9, src/Constants.cpp:80-88).
 * mifgpu_field_extent() reports them.
 *
 * Every entry point returns MIFGPU_OK (0) or a negative MIFGPU_E* code;
 * mifgpu_last_error() gives the message. A context is bound to the CUDA device
 * that was current at mifgpu_create() and to one stream; it is not thread-safe
 * (the reference's solver state is not re-entrant either,
 * src/PressureSolverStructures.cpp:13-70).
 *
 * Field ids (the reference's tensors passed to mif::timestep,
 * include/Timestep.h:16-19):
 *   0..2  velocity.{u,v,w}            3..5  velocity_buffer.{u,v,w}
 *   6..8  velocity_buffer_2.{u,v,w}   9     pressure
 *   10    pressure_buffer (the Poisson solution phi of the last solve)
 */
#ifndef MIFGPU_H
#define MIFGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MIFGPU_OK 0
#define MIFGPU_EINVAL (-1)   /* bad argument (null pointer, size, id, mode) */
#define MIFGPU_ECUDA (-2)    /* a CUDA call failed, a TMA tensor map was
                                rejected, or a kernel gave up waiting for a
                                TMA tile load (each wait is bounded); see
                                mifgpu_last_error */
#define MIFGPU_ENOMEM (-3)   /* device allocation failed */
#define MIFGPU_ENOTSUP (-4)  /* combination the reference does not define */
#define MIFGPU_ENONFINITE (-5) /* a projection step produced NaN/Inf: the last
                                  projection of every step checks each value
                                  of phi, which a NaN/Inf anywhere in the
                                  velocity reaches (mifgpu_timestep, _run,
                                  _timestep_host, _timestep_nhn; the fields
                                  hold the non-finite state) */

enum mifgpu_precision {
  MIFGPU_FP64 = 0,  /* everything in double: the reference's USE_DOUBLE=1 build */
  MIFGPU_MIXED = 1, /* fields and stencils in float; the eigenvalues and
                       1/(lx+ly+lz) computed in double and applied as a float
                       table; zero-mode handling and reductions in double;
                       the state updates round stochastically */
  MIFGPU_MIXED_COMPENSATED = 2 /* as MIXED, and every velocity component of the
                       state carries a bfloat16 residual: each state update
                       (RK stage, projection, boundary fill) is an error-free
                       float sum whose rounding error is kept in the residual,
                       and the divergence reads hi + residual, so the state is
                       held to about 32 significant bits while the stencils and
                       transforms still read float. Host transfers of velocity
                       set 0 and the error norms see hi + residual. The
                       velocity-only step and the reverse mode return
                       MIFGPU_ENOTSUP in this mode. Inside a step the Y3 and U*
                       stage kernels apply the projection before them, and in
                       a run of several steps each step's Y2 stage applies the
                       previous step's last projection (the run's last step
                       ends with it), so after a call velocity_buffer and
                       velocity_buffer_2 (scratch in the reference too) hold
                       unprojected stage states; the context holds two more
                       pressure-sized buffers. */
};

/* Analytic field families used for Dirichlet boundary data, forcing and
 * error norms (the reference passes them as std::function,
 * include/VectorFunction.h:33-53). */
enum mifgpu_field_kind {
  MIFGPU_FIELD_ZERO = 0,   /* no-slip walls / periodic boxes */
  MIFGPU_FIELD_SINCOS = 1, /* u = sin x cos y sin z sin t, v = cos x sin y sin z sin t,
                              w = 2 cos x cos y cos z sin t, p = cos x cos y sin z sin t
                              (generators/manufsol_velocity.py:55-57) */
  MIFGPU_FIELD_ETHIER = 2, /* exact NS solution of test/full_test.cpp
                              (generators/manufsol.py:35-72) */
  MIFGPU_FIELD_CALLER = 3  /* any exact velocity: the caller supplies the
                              Dirichlet face values of every stage
                              (mifgpu_set_boundary_values) and, for the
                              non-homogeneous Neumann step, the normal
                              pressure-gradient data
                              (mifgpu_set_pressure_gradient_faces). There is
                              no analytic field: set_exact_*, adjust_pressure,
                              the error norms and the reverse mode return
                              MIFGPU_ENOTSUP, and mifgpu_run takes one step
                              per call */
};

/* Forcing added to the momentum right-hand side of the projection step.
 * The reference's mif::timestep has none (src/Timestep.cpp:16,32,49); the
 * two others are extensions for manufactured-solution runs. */
enum mifgpu_forcing {
  MIFGPU_FORCING_NONE = 0,
  MIFGPU_FORCING_VELOCITY = 1,     /* u_t + (u.grad)u - lap(u)/Re of the SINCOS velocity,
                                      include/MomentumEquationForcing.h:10-32 */
  MIFGPU_FORCING_NAVIER_STOKES = 2, /* the same plus grad p of the SINCOS pressure */
  MIFGPU_FORCING_TAYLOR_GREEN = 3    /* alpha * (sin x cos y cos z, -cos x sin y cos z, 0),
                                        alpha = forcing_amplitude (a body force for the
                                        periodic-box gradient runs) */
};

typedef struct {
  long n_global[3];  /* points per axis, include/Constants.h:14-16: a periodic axis
                        with N unique points has N + 1; a Dirichlet axis counts
                        both walls */
  double size[3];    /* domain lengths (x_size, y_size_global, z_size_global) */
  double origin[3];  /* min_x_global, min_y_global, min_z_global */
  double Re;         /* Reynolds number */
  double dt;         /* time step (Constants::dt) */
  int periodic[3];   /* periodic_bc */
  int precision;     /* enum mifgpu_precision */
  int boundary_kind; /* enum mifgpu_field_kind: exact velocity on Dirichlet faces */
  int forcing;       /* enum mifgpu_forcing */
  double forcing_amplitude; /* alpha of MIFGPU_FORCING_TAYLOR_GREEN */
} mifgpu_params;

typedef struct mifgpu_ctx mifgpu_ctx;

/* Replaces the set-up of src/main.cpp:127-141: Constants,
 * PressureSolverStructures (src/PressureSolverStructures.cpp:13-70) and the
 * six tensors. All fields start at zero.
 * Returns MIFGPU_EINVAL, with *out left NULL and no device work done, for
 * parameters out of range:
 *   - fewer than 3 points on an axis;
 *   - a staggered extent above the CUDA grid limits of the box kernels,
 *     where the staggered extent is n_global + 1 on a Dirichlet axis and
 *     n_global + 2 on a periodic y or z axis: z above 65535, y above
 *     262140, any axis above 524280.
 * A Poisson line longer than the shared-memory transforms hold returns
 * MIFGPU_ENOTSUP with a context whose mifgpu_last_error() says so; the
 * caller destroys it. */
int mifgpu_create(const mifgpu_params *params, mifgpu_ctx **out);
int mifgpu_destroy(mifgpu_ctx *ctx);

/* Stream for every launch and copy (default: a stream the context creates).
 * `stream` is a cudaStream_t. */
int mifgpu_set_stream(mifgpu_ctx *ctx, void *stream);
int mifgpu_synchronize(mifgpu_ctx *ctx);
const char *mifgpu_last_error(const mifgpu_ctx *ctx);

/* Extents (Ex, Ey, Ez) of a field in the reference layout. */
int mifgpu_field_extent(const mifgpu_ctx *ctx, int field, long out[3]);

/* Host <-> device copies of one field in the reference layout (double).
 * upload is asynchronous on the context's stream: the host buffer must stay
 * valid until the next synchronising call. download returns after the data
 * has landed in `host`. The data travels as DMA copies of 64 MB chunks,
 * spread over four copy streams, into a device staging slot, and one layout
 * kernel (mifgpu_timestep_host queues its four fields this way at once, so
 * the copies of one field overlap the layout kernels of another). Measured
 * on GB300 with pinned buffers: ~210 GB/s host to device and ~192 GB/s
 * device to host, the link's per-direction rate for plain copies; kernels
 * reading host memory directly over NVLink-C2C were ~10% slower. */
int mifgpu_upload(mifgpu_ctx *ctx, int field, const double *host);
int mifgpu_download(mifgpu_ctx *ctx, int field, double *host);

/* Initial conditions from the analytic family (test/full_test.cpp:86-89):
 * velocity set `set` (0..2) sampled at time t on every point, or the pressure. */
int mifgpu_set_exact_velocity(mifgpu_ctx *ctx, int set, double t);
int mifgpu_set_exact_pressure(mifgpu_ctx *ctx, double t);

/* One projection step from t_n, replaces mif::timestep
 * (include/Timestep.h:16-19, src/Timestep.cpp:151-156). Works on the
 * device-resident fields. */
int mifgpu_timestep(mifgpu_ctx *ctx, double t_n);

/* `nsteps` projection steps from t0 with t_n = t0 + n*dt, replayed from one
 * captured CUDA graph (the loop of src/main.cpp:149-156). */
int mifgpu_run(mifgpu_ctx *ctx, double t0, int nsteps);

/* The drop-in form of mif::timestep for callers that keep the fields on the
 * host: uploads velocity (u,v,w) and pressure, steps, downloads them back.
 * Buffers are in the reference layout (extents of fields 0,1,2,9). */
int mifgpu_timestep_host(mifgpu_ctx *ctx, double t_n, double *u, double *v, double *w, double *p);

/* Non-homogeneous Neumann pressure variant, replaces mif::timestep_nhn
 * (src/Timestep.cpp:143-149); the pressure-gradient data is the gradient of
 * the boundary kind's pressure. Requires no periodic axis. */
int mifgpu_timestep_nhn(mifgpu_ctx *ctx, double t_n);

/* Velocity-only RK3 step with the SINCOS forcing, replaces
 * mif::timestep_velocity (src/TimestepVelocity.cpp:60-90): uses sets 0..2 as
 * velocity, velocity_buffer and rhs_buffer, and ends with the swap of
 * src/TimestepVelocity.cpp:89. */
int mifgpu_timestep_velocity(mifgpu_ctx *ctx, double t_n);

/* `nsteps` velocity-only steps from t0 with t_n = t0 + n*dt, each ending with
 * the swap, replayed from the captured graphs of the two labellings with no
 * host synchronisation between steps: the loop of the reference's benchmark
 * harness over mif::timestep_velocity (test/benchmark.cpp:42-50). */
int mifgpu_run_velocity(mifgpu_ctx *ctx, double t0, int nsteps);

/* Sub-steps, for parity testing and for callers that assemble their own step:
 *   apply_bc       VelocityTensor::apply_bc on set `set` at time t
 *                  (src/VelocityTensor.cpp:36-233)
 *   solve_pressure solve_pressure_equation_homogeneous_periodic: phi from
 *                  div(set)/dt (src/PressureEquation.cpp:266-274)
 *   divergence     phi := div(set)/dt on owner points only
 *                  (src/PressureEquation.cpp:59-61)
 *   project        p += phi and set -= dt * grad(phi) on interior points
 *                  (src/Timestep.cpp:66-81) */
int mifgpu_apply_bc(mifgpu_ctx *ctx, int set, double t);

/* Caller boundary data for boundary_kind MIFGPU_FIELD_CALLER. Replaces the
 * evaluation of the caller's exact_velocity inside the step
 * (VelocityTensor::apply_bc, src/VelocityTensor.cpp:36-233, called by
 * src/Timestep.cpp:110,120,130 with exact_velocity.set_time(t_k)). u, v, w are
 * host arrays in the reference layout (extents of fields 0, 1, 2); only their
 * Dirichlet face planes are read: the values apply_bc writes there at the
 * slot's time (a caller gets them by running the reference's own apply_bc on
 * a scratch VelocityTensor). Slot 0 is what mifgpu_apply_bc imposes; slots 1,
 * 2, 3 are the stage times time_1, time_2, final_time of the next
 * mifgpu_timestep / _timestep_host / _timestep_nhn / _run(ctx, t, 1) (and of
 * mifgpu_timestep_velocity's stages). Copied at the call; a slot keeps its
 * data until set again (all zero at first). */
int mifgpu_set_boundary_values(mifgpu_ctx *ctx, int slot, const double *u, const double *v, const double *w);

/* Caller data of the non-homogeneous Neumann step (MIFGPU_FIELD_CALLER):
 * replaces exact_pressure_gradient.get_difference_over_time(t_k, t_{k-1}) of
 * src/Timestep.cpp:85-90, i.e. grad p(t_{k-1}) - grad p(t_k), for stage k =
 * slot (1..3; slot 0 is overwritten by mifgpu_solve_pressure_nhn). faces[f]
 * holds the normal component on face f = x_min, x_max, y_min, y_max, z_min,
 * z_max at the face's pressure nodes, the two other axes in order, lower one
 * fastest: (j, k) -> j + Ny k on x faces, (i, k) -> i + Nx k on y faces,
 * (i, j) -> i + Nx j on z faces (Nx, Ny: the pressure extents). Copied at the
 * call. */
int mifgpu_set_pressure_gradient_faces(mifgpu_ctx *ctx, int slot, const double *const faces[6]);

/* solve_pressure_equation_non_homogeneous_neumann (include/PressureEquation.h:15-19,
 * src/PressureEquation.cpp:276-286): phi := div(set)/dt plus the boundary
 * terms of apply_non_homogeneous_neumann (src/PressureEquation.cpp:10-56)
 * from `faces` (the normal component of the caller's exact_pressure_gradient
 * at the face nodes, laid out as for mifgpu_set_pressure_gradient_faces),
 * then the spectral solve. Any boundary kind; every axis must be
 * non-periodic (MIFGPU_ENOTSUP otherwise). */
int mifgpu_solve_pressure_nhn(mifgpu_ctx *ctx, int set, double dt, const double *const faces[6]);
int mifgpu_solve_pressure(mifgpu_ctx *ctx, int set, double dt);
int mifgpu_divergence(mifgpu_ctx *ctx, int set, double dt);
int mifgpu_project(mifgpu_ctx *ctx, int set, double dt);

/* Mean shift of the pressure towards the boundary kind's exact pressure at t
 * (adjust_pressure, src/PressureEquation.cpp:288-343), in double. */
int mifgpu_adjust_pressure(mifgpu_ctx *ctx, double t);

/* The nine numbers of test/full_test.cpp:150-175 against the boundary kind's
 * exact fields at t: L1, L2, Linf of velocity, pressure, pressure gradient
 * (src/Norms.cpp:11-118). Reductions in double. */
int mifgpu_error_norms(mifgpu_ctx *ctx, double t, double out[9]);

/* The reference's writers on velocity set 0 and the pressure
 * (include/VTKDatExport.h:10-29, src/VTKDatExport.cpp), for one rank, with
 * the reference's byte layouts; values are computed in the context's
 * precision (double for MIFGPU_FP64, float for MIFGPU_MIXED, as the
 * reference's Real), from the planes or lines fetched off the device:
 *   write_vtk            planes x = 0, y = 0, z = 0, velocity interpolated
 *                        to the pressure points and the pressure, binary
 *                        big-endian unstructured-grid VTK (writeVTK); x = 0
 *                        must lie in the domain (the reference asserts it)
 *   write_dat            the profile line parallel to axis `direction`
 *                        (0 x, 1 y, 2 z) through (x, y, z), which must lie on
 *                        pressure planes or midway between them (writeDat)
 *   write_vtk_full_mesh  every pressure point, ASCII VTK (writeVTKFullMesh) */
int mifgpu_write_vtk(mifgpu_ctx *ctx, const char *filename);
int mifgpu_write_dat(mifgpu_ctx *ctx, const char *filename, int direction, double x, double y, double z);
int mifgpu_write_vtk_full_mesh(mifgpu_ctx *ctx, const char *filename);

/* Kernel classes of one projection step, for mifgpu_profile_step. */
enum mifgpu_prof_class {
  MIFGPU_PROF_STAGE = 0,      /* the three fused RK stage updates */
  MIFGPU_PROF_BOUNDARY = 1,   /* Dirichlet faces + periodic copies of the velocity */
  MIFGPU_PROF_DIVERGENCE = 2, /* Poisson right-hand side */
  MIFGPU_PROF_X_FORWARD = 3,  /* line transforms: x forward */
  MIFGPU_PROF_Y_FORWARD = 4,  /* y forward */
  MIFGPU_PROF_Z_FUSED = 5,    /* z forward, eigenvalue division, z inverse */
  MIFGPU_PROF_Y_INVERSE = 6,  /* y inverse */
  MIFGPU_PROF_X_INVERSE = 7,  /* x inverse */
  MIFGPU_PROF_PERIODIC = 8,   /* periodic refresh of phi */
  MIFGPU_PROF_PROJECT = 9,    /* p += phi, u -= dt grad phi */
  MIFGPU_PROF_CLASSES = 10
};

/* Runs `reps` projection steps from t_n launch by launch (not from the graph),
 * timing every kernel class with CUDA events on the context's stream; writes
 * the mean milliseconds per step of each class. The steps are real: the
 * fields advance. In MIFGPU_MIXED_COMPENSATED the timed step is the one a
 * run of several steps repeats (its Y2 stage applies the previous step's last
 * projection; no projection kernel of its own), with one untimed step before
 * and one after. No counterpart in the reference (instrumentation). */
int mifgpu_profile_step(mifgpu_ctx *ctx, double t_n, int reps, double ms_out[MIFGPU_PROF_CLASSES]);

/* ---- Reverse mode (no counterpart in the reference) ----
 *
 * Discrete adjoint of `nsteps` projection steps of mifgpu_run from the
 * context's current state at t0 (velocity set 0 and the pressure are the
 * inputs; sets 1, 2 and phi are scratch, as in the reference). The forward
 * pass stores (u, v, w, p) every `checkpoint_every` steps (1..1024); the
 * backward pass recomputes one segment at a time, keeping the three sets each
 * stage's right-hand side was evaluated at, and runs the transposed step
 * kernels in reverse. Device memory: 11 adjoint fields + 4 per checkpoint
 * (nsteps / checkpoint_every + 2 of them) + 9 per step of a segment.
 *
 * On return the context holds the final state, and mifgpu_download_adjoint
 * gives d loss / d (initial field) for field ids 0, 1, 2 (u, v, w of set 0,
 * every point of their extents, ghosts included) and 9 (pressure).
 * `dloss_dalpha` (may be null) receives the derivative with respect to
 * forcing_amplitude when the forcing is MIFGPU_FORCING_TAYLOR_GREEN, else 0.
 * The backward pass recomputes each segment on a second stream into one of
 * two snapshot buffers, so the recompute of a segment runs beside the reverse
 * sweep of the one after it (with one buffer, when two do not fit, they
 * alternate). `ms_out` (may be null) receives milliseconds, timed with CUDA
 * events: [0] the forward pass, [1] the whole backward pass (seed,
 * recomputes and reverse sweeps, wall time), [2] the reverse sweeps alone
 * (summed over the segments on the reverse stream; they share the GPU with
 * the recomputes beside them). */

/* Loss = 1/2 hx hy hz * sum of u_c^2 over the interior staggered points of
 * each component whose position lies in box = {x0, x1, y0, y1, z0, z1}
 * (the kinetic energy in a sub-box at the final time). */
int mifgpu_gradient_ke(mifgpu_ctx *ctx, double t0, int nsteps, int checkpoint_every, const double box[6],
                       double *loss, double *dloss_dalpha, double ms_out[3]);

/* The same for a caller-defined loss: seed_{u,v,w,p} are d loss / d (final
 * field) in the reference layout (null = zero). */
int mifgpu_backward(mifgpu_ctx *ctx, double t0, int nsteps, int checkpoint_every, const double *seed_u,
                    const double *seed_v, const double *seed_w, const double *seed_p, double *dloss_dalpha,
                    double ms_out[3]);

/* d loss / d (initial field) of the last mifgpu_gradient_ke / mifgpu_backward. */
int mifgpu_download_adjoint(mifgpu_ctx *ctx, int field, double *host);

/* Changes alpha of the Taylor-Green forcing (re-captures the step graphs). */
int mifgpu_set_forcing_amplitude(mifgpu_ctx *ctx, double alpha);

/* Velocity error norms that allocate nothing. No counterpart in the
 * reference: it is a variant of the velocity part of mifgpu_error_norms
 * (out[0..2] = L1, L2, Linf of velocity set 0 against the boundary kind's
 * exact velocity at t, src/Norms.cpp:11-47) for callers that cannot allocate
 * device memory in the middle of a run: a time loop that has handed the rest
 * of HBM to a caching allocator (PyTorch's, for one), where a lazy cudaMalloc
 * fails with out-of-memory, and loops that cannot take the device-wide
 * synchronisation cudaMalloc/cudaFree imply.
 *
 * Its partial sums live in one file-scope device array of the library
 * (96 KB: 3 doubles for each of at most 4000 interior z planes, plus the
 * totals); nothing in it has to start at zero, because every element the call
 * reads it has written before. The reduction runs in a fixed order, so the
 * result is bitwise reproducible. The call returns MIFGPU_EINVAL, with a
 * message, for more than 4000 interior z planes, that is n_global[2] above
 * 4002 on a Dirichlet z axis or above 4001 on a periodic one, and when the
 * context's device is not the current device. The first call on a device
 * (and the first after its context was re-created, e.g. by cudaDeviceReset)
 * looks up the array's address (cudaGetSymbolAddress) and caches it; make
 * that first call before any stream capture begins on the device. In the
 * compensated precision the velocity is read as hi + residual, as in
 * mifgpu_error_norms. The array is shared by every context on a device: calls whose
 * executions overlap (other threads, other streams or contexts on the same
 * device) race on it, so the caller serialises them. Returns after the three
 * numbers have reached `out`. */
int mifgpu_velocity_error_norms_noalloc(mifgpu_ctx *ctx, double t, double out[3]);

/* Number of kernels this context has launched so far (for launch accounting). */
int mifgpu_launch_count(const mifgpu_ctx *ctx, long long *out);

/* Device bytes held by the context. */
int mifgpu_device_bytes(const mifgpu_ctx *ctx, size_t *out);

/* No counterpart in the reference (instrumentation). The FP64 fused
 * multiply-add rate of the current device in TFLOP/s (an FMA counted as two
 * operations): independent FMA chains on every SM, timed with CUDA events
 * after one warm-up launch. It is the FP64-pipe ceiling of a plain FP64 step,
 * beside the HBM one. Needs no context; synchronises the device. */
int mifgpu_probe_fp64_fma(double *tflops);

#ifdef __cplusplus
}
#endif

#endif /* MIFGPU_H */
