// Host launchers of the point-wise kernels (stencil.cu).
#pragma once

#include "common.cuh"

namespace mifgpu {

// Device pointers of the eleven fields of a context, in the working precision.
template <typename T>
struct Fields {
  T *f[kNumFields];
  __host__ __device__ T *vel(int set, int c) const { return f[set * kFieldsPerSet + c]; }
};

enum StageKind {
  kStageY2 = 0,     // src/Timestep.cpp:10-21
  kStageY3 = 1,     // src/Timestep.cpp:24-39
  kStageUStar = 2,  // src/Timestep.cpp:42-54
  kVelY2 = 3,       // src/TimestepVelocity.cpp:20-29
  kVelY3 = 4,       // src/TimestepVelocity.cpp:32-42
  kVelUStar = 5     // src/TimestepVelocity.cpp:45-52
};

// Forcing tables: sin and cos of every node and face coordinate per axis,
// evaluated on the host (libm, double) and stored in T.
template <typename T>
struct ForcingTables {
  const T *tab = nullptr;  // [axis][0 node / 1 face][0 sin / 1 cos][maxE]
  int maxE = 0;
};

// Stage times live in device memory so that a captured CUDA graph can be
// replayed step after step: slot s of step n is slots[n * kSlotSize + s] with
// n = *step. Layout of one step's slot (doubles):
//   0 t_n, 1 time_1, 2 time_2, 3 final time,
//   4/5 sin/cos(t_n), 6/7 sin/cos(time_1), 8/9 sin/cos(time_2),
//   10..13 the velocity family's time factor at times 0..3,
//   14..17 the pressure-gradient family's time factor at times 0..3
// (both families are a spatial field times a factor of t; see FaceTables).
constexpr int kSlotSize = 18;
constexpr int kSlotFactor = 10;
struct TimeRef {
  const double *slots;
  const int *step;
  __device__ __forceinline__ double get(int s) const { return slots[(long)(*step) * kSlotSize + s]; }
};

// Dirichlet face data in double. Two uses:
// - analytic families, precomputed at a unit time for the float path:
//   value(x, t) = tab[...](x) * factor(t), with the factor in the time slots;
// - caller data (MIFGPU_FIELD_CALLER, slot_stride > 0): the values the
//   reference's apply_bc writes, one table per time slot at
//   tab + slot * slot_stride, used as they are.
// off[fn][c][d][s] is the start of the table of family fn (0 velocity, 1
// pressure gradient), component c, faces normal to axis d, side s; the face
// point (pa, pb) (the two other axes, in order) is at pa + ext(c, a) * pb.
// A null tab means: evaluate in the working precision.
struct FaceTables {
  const double *tab = nullptr;
  long off[2][3][3][2] = {};
  long slot_stride = 0;
};

// Caller-supplied normal pressure-gradient data of the non-homogeneous
// Neumann problem, one table per time slot at tab + slot * slot_stride: the
// six faces x_min, x_max, y_min, y_max, z_min, z_max at off[f], each over the
// pressure nodes of the face, (j, k) -> j + E1 k on x faces, (i, k) -> i + E0 k
// on y faces, (i, j) -> i + E0 j on z faces.
struct GradFaces {
  const double *tab = nullptr;
  long off[6] = {};
  long slot_stride = 0;
};

template <typename T>
struct StageScalars {
  double dt;     // Constants::dt
  int sin_slot;  // slot of sin(stage time); cos follows it
  int forcing;   // 0 none, 1 velocity forcing, 2 with grad p, 3 Taylor-Green body force
  double alpha;  // amplitude of the Taylor-Green body force
};

// The projection that precedes a compensated stage, applied by the stage
// kernel itself (see stage_proj_kernel): phi of the previous solve, the
// pressure read (p_in) and written as p + phi (p_out, another buffer), and the
// previous projection's dt and stochastic-rounding tag (launch_project's).
struct StageProj {
  const float *phi = nullptr;
  const float *p_in = nullptr;
  float *p_out = nullptr;
  float dt = 0.f;
  unsigned tag = 0;
};

// `res`: the compensated state's residuals (projection stages, float only).
// `proj` (compensated projection stages only, or null): the preceding
// projection, done inside the stage. The plane ring is filled by TMA tile
// loads; `kerr` (device, may be null) is set to 1 if a CTA gave up waiting
// for one. Returns false (nothing launched) if a tensor map was rejected.
template <typename T>
bool launch_stage(const Geometry &g, const Fields<T> &F, StageKind st, const StageScalars<T> &sc,
                  const ForcingTables<T> &ft, int field_kind, TimeRef tr, cudaStream_t s, long long *launches,
                  const Residual &res = Residual{}, const StageProj *proj = nullptr, int *kerr = nullptr);

// Dirichlet faces (fn 0 velocity family, 1 pressure-gradient family) then the
// periodic copies, on velocity set `set` (src/VelocityTensor.cpp:36-233).
// With `res` on, the faces are written as hi + residual and the periodic
// copies carry the residual along.
template <typename T>
void launch_apply_bc(const Geometry &g, T *const comp[3], int field_kind, int fn, TimeRef tr, int t_slot,
                     const FaceTables &ft, cudaStream_t s, long long *launches, const Residual &res = Residual{});

// Fills the face tables of family fn (see FaceTables) in double.
void launch_face_tables(const Geometry &g, int field_kind, int fn, double *tab, const FaceTables &ft,
                        cudaStream_t s);

// Time factor of family fn (0 velocity, 1 pressure gradient) at time t, and
// the unit time at which the tables are evaluated.
double family_time_factor(int field_kind, int fn, double t, double Re);
double family_unit_time(int field_kind);

// Periodic ghost copy of a pressure-shaped field (src/StaggeredTensor.cpp:221-257).
template <typename T>
void launch_periodic_scalar(const Geometry &g, T *f, cudaStream_t s, long long *launches);

// phi := div(vel)/dt on owner points (src/PressureEquation.cpp:59-61).
template <typename T>
void launch_divergence(const Geometry &g, T *phi, T *const vel[3], double dt, cudaStream_t s, long long *launches,
                       const Residual &res = Residual{});

// phi += boundary flux terms of the non-homogeneous Neumann problem
// (src/PressureEquation.cpp:10-56), data = grad p(t_old) - grad p(t_new).
template <typename T>
void launch_neumann_flux(const Geometry &g, T *phi, int field_kind, TimeRef tr, int slot_new, int slot_old,
                         cudaStream_t s, long long *launches);

// The same flux terms from caller data: phi += 2 G / h on every boundary node
// for each face holding it, in the reference's face order, with G the
// GradFaces table of time slot `slot` (src/PressureEquation.cpp:10-56).
template <typename T>
void launch_neumann_flux_data(const Geometry &g, T *phi, const GradFaces &gf, int slot, cudaStream_t s,
                              long long *launches);

// p += phi everywhere; vel -= dt * grad(phi) on interior points (src/Timestep.cpp:66-81).
// In float both updates round stochastically, drawn from the step time in
// tr's slot 0 and `tag` (one per projection of a step).
// With `res` on (float), the velocity update is an error-free sum into hi + residual.
// `nonfinite` (may be null) is set to 1 if any phi value is NaN or Inf.
template <typename T>
void launch_project(const Geometry &g, T *p, const T *phi, T *const vel[3], double dt, TimeRef tr, unsigned tag,
                    cudaStream_t s, long long *launches, const Residual &res = Residual{}, int *nonfinite = nullptr);

// Reference layout (double, contiguous) <-> device layout (T, padded); `lo`:
// the field's residual array in the compensated state (split on the way in,
// added on the way out), or null.
template <typename T>
void launch_scatter(const Geometry &g, T *dst, const double *src, int ex, int ey, int ez, cudaStream_t s,
                    long long *launches, __nv_bfloat16 *lo = nullptr);
template <typename T>
void launch_gather(const Geometry &g, double *dst, const T *src, int ex, int ey, int ez, cudaStream_t s,
                   long long *launches, const __nv_bfloat16 *lo = nullptr);

// Analytic initial fields (every point): comp 0..2 velocity component of a
// set, 3 pressure.
template <typename T>
void launch_set_exact(const Geometry &g, T *f, int comp, int field_kind, double t, cudaStream_t s,
                      long long *launches, __nv_bfloat16 *lo = nullptr);

// Sum of (exact p - p) over owner points into *acc (double, device).
template <typename T>
void launch_pressure_mean_diff(const Geometry &g, const T *p, int field_kind, double t, double *acc,
                               cudaStream_t s, long long *launches);
// p += *shift on every point.
template <typename T>
void launch_add_scalar(const Geometry &g, T *p, const double *shift, cudaStream_t s, long long *launches);

// Error accumulators in double: acc[0] sum |e|-norm, acc[1] sum e^2, acc[2] max.
template <typename T>
void launch_velocity_errors(const Geometry &g, T *const vel[3], int field_kind, int fn, double t, double *acc,
                            cudaStream_t s, long long *launches, const Residual &res = Residual{});
template <typename T>
void launch_pressure_errors(const Geometry &g, const T *p, int field_kind, double t, double *acc, cudaStream_t s,
                            long long *launches);
// gradient of p into the interior of vel (src/PressureGradient.h:9-24)
template <typename T>
void launch_pressure_gradient(const Geometry &g, T *const vel[3], const T *p, cudaStream_t s, long long *launches);

}  // namespace mifgpu
