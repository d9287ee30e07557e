// C ABI of mifgpu (include/mifgpu.h): context set-up, host transfers, and the
// orchestration of one projection step as a single captured CUDA graph.
//
// Step structure (src/Timestep.cpp:97-141), all on the context's stream:
//   for each stage k: stage update -> boundary fill -> divergence ->
//   Poisson solve (5 line sweeps) -> periodic refresh of phi -> projection
// Stage times are read by the kernels from a device slot array, so one graph
// replays every step of a run without re-capture.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/mifgpu.h"
#include "adjoint_impl.cuh"
#include "common.cuh"
#include "export.cuh"
#include "noalloc.cuh"
#include "poisson.cuh"
#include "stencil.cuh"

using namespace mifgpu;

namespace {

// One reverse-mode request: nsteps projection steps from the context's
// state at t0, a loss on the final state, and its back-propagation.
struct GradRequest {
  double t0 = 0;
  int nsteps = 0;
  int every = 1;                                        // checkpoint interval (steps)
  const double *box = nullptr;                          // kinetic-energy loss box, or null
  const double *seed[4] = {nullptr, nullptr, nullptr, nullptr};  // host d loss / d (u, v, w, p) otherwise
  double *loss = nullptr, *dalpha = nullptr, *ms = nullptr;
};

struct ImplBase {
  virtual ~ImplBase() = default;
  virtual int init(mifgpu_ctx *ctx) = 0;
  virtual void *field_ptr(int id) = 0;
  virtual int upload(mifgpu_ctx *ctx, int id, const double *host) = 0;
  virtual int download(mifgpu_ctx *ctx, int id, double *host) = 0;
  virtual int upload_fields(mifgpu_ctx *ctx, const int *ids, const double *const *host, int count) = 0;
  virtual int download_fields(mifgpu_ctx *ctx, const int *ids, double *const *host, int count) = 0;
  virtual int set_exact(mifgpu_ctx *ctx, int id, double t) = 0;
  virtual int step(mifgpu_ctx *ctx, int variant, const double *slots, int nsteps) = 0;
  virtual int apply_bc(mifgpu_ctx *ctx, int set, double t) = 0;
  virtual int solve_pressure(mifgpu_ctx *ctx, int set, double dt, bool solve) = 0;
  virtual int project(mifgpu_ctx *ctx, int set, double dt) = 0;
  virtual int adjust_pressure(mifgpu_ctx *ctx, double t) = 0;
  virtual int error_norms(mifgpu_ctx *ctx, double t, double out[9]) = 0;
  virtual int profile_step(mifgpu_ctx *ctx, double t_n, int reps, double *ms) = 0;
  virtual void swap_sets() = 0;
  virtual size_t bytes() const = 0;
  virtual int gradient(mifgpu_ctx *ctx, const GradRequest &req) = 0;
  virtual int download_adjoint(mifgpu_ctx *ctx, int id, double *host) = 0;
  virtual void drop_graphs() = 0;
  virtual int fetch_box(mifgpu_ctx *ctx, int id, const int lo[3], const int n[3], double *out) = 0;
  // The compensated state's residuals (off unless MIFGPU_MIXED_COMPENSATED).
  virtual Residual residual() const = 0;
  // Caller boundary data (MIFGPU_FIELD_CALLER) and the stand-alone
  // non-homogeneous Neumann solve.
  virtual int set_boundary_values(mifgpu_ctx *ctx, int slot, const double *const vel[3]) = 0;
  virtual int set_gradient_faces(mifgpu_ctx *ctx, int slot, const double *const faces[6]) = 0;
  virtual int solve_pressure_nhn(mifgpu_ctx *ctx, int set, double dt) = 0;
};

}  // namespace

struct mifgpu_ctx {
  mifgpu_params prm{};
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  Geometry g{};
  std::string err;
  long long launches = 0;
  std::unique_ptr<ImplBase> impl;
};

namespace {

int fail(mifgpu_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int cuda_fail(mifgpu_ctx *ctx, cudaError_t e, const char *where) {
  return fail(ctx, MIFGPU_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

// Extents of field id in the reference layout.
void field_extent(const Geometry &g, int id, int e[3]) {
  if (id < 9) {
    const int c = id % 3;
    for (int d = 0; d < 3; ++d) e[d] = g.ext(c, d);
  } else {
    for (int d = 0; d < 3; ++d) e[d] = g.E[d];
  }
}

// Time factors of the analytic families at the slot's four times.
void slot_factors(double *s, int kind, double Re) {
  for (int q = 0; q < 4; ++q) {
    s[kSlotFactor + q] = family_time_factor(kind, 0, s[q], Re);
    s[kSlotFactor + 4 + q] = family_time_factor(kind, 1, s[q], Re);
  }
}

// Times of one projection step, computed as src/Timestep.cpp:97-104 does.
void projection_slot(double t_n, double dt, int kind, double Re, double *s) {
  const double dt_1 = 64.0 / 120.0 * dt;
  const double time_1 = t_n + dt_1;
  const double dt_2 = 16.0 / 120.0 * dt;
  const double time_2 = time_1 + dt_2;
  const double final_time = t_n + dt;
  s[0] = t_n;
  s[1] = time_1;
  s[2] = time_2;
  s[3] = final_time;
  s[4] = std::sin(t_n);
  s[5] = std::cos(t_n);
  s[6] = std::sin(time_1);
  s[7] = std::cos(time_1);
  s[8] = std::sin(time_2);
  s[9] = std::cos(time_2);
  slot_factors(s, kind, Re);
}

// Times of one velocity-only step, src/TimestepVelocity.cpp:63-65.
void velocity_slot(double t_n, double dt, int kind, double Re, double *s) {
  const double c2 = (8.0 / 15.0), c3 = (2.0 / 3.0);
  const double time_1 = t_n + c2 * dt;
  const double time_2 = t_n + c3 * dt;
  const double final_time = t_n + dt;
  s[0] = t_n;
  s[1] = time_1;
  s[2] = time_2;
  s[3] = final_time;
  s[4] = std::sin(t_n);
  s[5] = std::cos(t_n);
  s[6] = std::sin(time_1);
  s[7] = std::cos(time_1);
  s[8] = std::sin(time_2);
  s[9] = std::cos(time_2);
  slot_factors(s, kind, Re);
}

enum { kVariantProjection = 0, kVariantNhn = 1, kVariantVelocity = 2 };

// Field values on an index box, converted to double, x fastest (the export writers' fetch).
template <typename T>
__global__ void box_gather_kernel(Geometry g, double *dst, const T *src, int lo0, int lo1, int lo2, int n0, int n1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= n0 || j >= n1) return;
  dst[i + (long)n0 * (j + (long)n1 * k)] = (double)src[g.idx(lo0 + i, lo1 + j, lo2 + k)];
}

// Last node of every captured step: the next replay reads the next time slot.
__global__ void advance_step_kernel(int *ctr) { *ctr += 1; }

template <typename T>
struct Impl final : ImplBase {
  Geometry g{};
  size_t field_elems = 0;
  T *block = nullptr;
  Fields<T> phys{};  // physical field pointers
  int parity = 0;    // 1 after an odd number of velocity-only steps: sets 0 and 1 exchanged
  Fields<T> F{};     // logical view (reference field ids) for the current parity
  PoissonSolver<T> ps{};
  T *ftab = nullptr;
  int ftab_maxE = 0;
  double *slots = nullptr;  // device: kSlotSize doubles per step
  int slots_cap = 0;
  int *step_ctr = nullptr;  // device step index the graph reads and advances
  // device flags: [0] a projection saw a NaN or Inf in phi, [1] a stage or
  // line kernel gave up waiting for a TMA tile load
  int *nonfinite = nullptr;
  double *acc = nullptr;    // device reduction scratch
  double *staging = nullptr;
  size_t staging_elems = 0;
  // Host transfers of several fields at once (mifgpu_timestep_host): one
  // reference-layout slot per field (slot 0 is `staging`), and copy streams
  // that split each field's copy into chunks so several copy engines run at
  // once while the scatter / gather kernels of other fields proceed.
  static constexpr int kXferSlots = 4, kCopyStreams = 4;
  double *xfer[kXferSlots] = {nullptr, nullptr, nullptr, nullptr};
  size_t xfer_elems = 0;
  cudaStream_t copy_stream[kCopyStreams] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t xfer_ev[kXferSlots + 1][kCopyStreams] = {};
  T *grad_block = nullptr;  // three fields for the pressure-gradient norm
  // MIFGPU_MIXED_COMPENSATED: the bfloat16 residuals of the velocity state
  // (one triple shared by the three sets, see Residual).
  __nv_bfloat16 *res_block = nullptr;
  Residual res{};
  // ... and the second pressure buffer of the stages that apply the preceding
  // projection themselves (StageProj: the Y3 stage writes p + phi here, the
  // U* stage reads it and writes the pressure field).
  T *p_alt = nullptr;
  // ... and a third one: within a run of several steps the Y2 stage applies
  // the previous step's last projection too, and the pressure cycles
  // p -> p_alt (Y2) -> p_alt2 (Y3) -> p (U*).
  T *p_alt2 = nullptr;
  double *face_tab = nullptr;  // float path: the families' face data in double; or the caller's
  FaceTables ftabs{};
  // Caller pressure-gradient face data (slots 0..3), allocated on first use.
  double *grad_tab = nullptr;
  GradFaces gfaces{};
  std::vector<double> pack;  // host packing buffer of the caller data
  cudaStream_t cap_stream = nullptr;
  // Step graphs per variant, labelling parity and phase (kPhase*).
  cudaGraphExec_t graph[3][2][4] = {};
  long long graph_launches[3][2][4] = {};
  size_t total_bytes = 0;
  // Per-kernel-class event marks of a profiled (non-graph) step.
  std::vector<std::pair<int, cudaEvent_t>> *prof = nullptr;
  // Reverse mode: the adjoint fields (lx 3, mu 3, pend 3, rho, lp), the
  // checkpoints (u, v, w, p per segment start and the final state) and the
  // per-step snapshots of one segment (the three sets each stage's
  // right-hand side was evaluated at).
  T *adj_block = nullptr;
  T *ckpt_block = nullptr;
  size_t ckpt_fields = 0;
  T *snap_block = nullptr;
  size_t snap_fields = 0;
  double *red_part = nullptr;  // per-block partial sums of the adjoint reductions
  // One captured reverse step per snapshot slot (the slot's address is baked in).
  std::vector<cudaGraphExec_t> rev_graph;
  long long rev_graph_launches = 0;
  // The backward pass's second stream (segment recomputes) and the events
  // that hand each of the two snapshot buffers between the streams.
  cudaStream_t rec_stream = nullptr;
  cudaEvent_t ev_rec[2] = {nullptr, nullptr}, ev_rev[2] = {nullptr, nullptr};

  void mark(int cls, cudaStream_t s) {
    if (!prof) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    prof->push_back({cls, e});
  }

  ~Impl() override {
    for (auto &gv : graph)
      for (auto &gp : gv)
        for (auto &gx : gp)
          if (gx) cudaGraphExecDestroy(gx);
    ps.release();
    cudaFree(block);
    cudaFree(ftab);
    cudaFree(slots);
    cudaFree(step_ctr);
    cudaFree(nonfinite);
    cudaFree(acc);
    cudaFree(staging);
    cudaFree(grad_block);
    cudaFree(res_block);
    cudaFree(p_alt);
    cudaFree(p_alt2);
    cudaFree(face_tab);
    cudaFree(grad_tab);
    cudaFree(adj_block);
    cudaFree(ckpt_block);
    cudaFree(snap_block);
    cudaFree(red_part);
    for (auto &gx : rev_graph)
      if (gx) cudaGraphExecDestroy(gx);
    if (cap_stream) cudaStreamDestroy(cap_stream);
    if (rec_stream) cudaStreamDestroy(rec_stream);
    for (int b = 0; b < 2; ++b) {
      if (ev_rec[b]) cudaEventDestroy(ev_rec[b]);
      if (ev_rev[b]) cudaEventDestroy(ev_rev[b]);
    }
    for (int q = 1; q < kXferSlots; ++q) cudaFree(xfer[q]);
    for (auto &row : xfer_ev)
      for (auto &e : row)
        if (e) cudaEventDestroy(e);
    for (auto &cs : copy_stream)
      if (cs) cudaStreamDestroy(cs);
  }

  int init(mifgpu_ctx *ctx) override {
    g = ctx->g;
    field_elems = (size_t)g.PX * g.PY * g.PZ;
    cudaError_t e = cudaMalloc(&block, sizeof(T) * field_elems * kNumFields);
    if (e != cudaSuccess) return fail(ctx, MIFGPU_ENOMEM, "cudaMalloc of the field block failed");
    total_bytes += sizeof(T) * field_elems * kNumFields;
    CK(cudaMemset(block, 0, sizeof(T) * field_elems * kNumFields));
    for (int f = 0; f < kNumFields; ++f) phys.f[f] = block + f * field_elems;
    remap();
    if (ctx->prm.precision == MIFGPU_MIXED_COMPENSATED) {
      if (cudaMalloc(&res_block, sizeof(__nv_bfloat16) * field_elems * 3) != cudaSuccess)
        return fail(ctx, MIFGPU_ENOMEM, "cudaMalloc of the residual fields failed");
      total_bytes += sizeof(__nv_bfloat16) * field_elems * 3;
      CK(cudaMemset(res_block, 0, sizeof(__nv_bfloat16) * field_elems * 3));
      for (int c = 0; c < 3; ++c) res.c[c] = res_block + c * field_elems;
      if (cudaMalloc(&p_alt, sizeof(T) * field_elems) != cudaSuccess ||
          cudaMalloc(&p_alt2, sizeof(T) * field_elems) != cudaSuccess)
        return fail(ctx, MIFGPU_ENOMEM, "cudaMalloc of the extra pressure buffers failed");
      total_bytes += 2 * sizeof(T) * field_elems;
      CK(cudaMemset(p_alt, 0, sizeof(T) * field_elems));
      CK(cudaMemset(p_alt2, 0, sizeof(T) * field_elems));
    }
    std::string perr;
    const int rc = ps.init(g, perr);
    if (rc) return fail(ctx, rc == -2 ? MIFGPU_ECUDA : MIFGPU_ENOTSUP, perr);
    // Forcing tables: sin/cos at nodes and faces of each axis (host libm, double).
    ftab_maxE = std::max({g.Es[0], g.Es[1], g.Es[2]}) + 1;
    std::vector<T> tab((size_t)3 * 2 * 2 * ftab_maxE);
    for (int ax = 0; ax < 3; ++ax)
      for (int face = 0; face < 2; ++face)
        for (int i = 0; i < ftab_maxE; ++i) {
          const double x = face ? g.face(ax, i) : g.node(ax, i);
          tab[((ax * 2 + face) * 2 + 0) * ftab_maxE + i] = T(std::sin(x));
          tab[((ax * 2 + face) * 2 + 1) * ftab_maxE + i] = T(std::cos(x));
        }
    CK(cudaMalloc(&ftab, sizeof(T) * tab.size()));
    CK(cudaMemcpy(ftab, tab.data(), sizeof(T) * tab.size(), cudaMemcpyHostToDevice));
    if (int rc = init_face_tables(ctx)) return rc;
    CK(cudaMalloc(&step_ctr, sizeof(int)));
    CK(cudaMemset(step_ctr, 0, sizeof(int)));
    CK(cudaMalloc(&nonfinite, 2 * sizeof(int)));
    CK(cudaMemset(nonfinite, 0, 2 * sizeof(int)));
    ps.err_flag = nonfinite + 1;
    CK(cudaMalloc(&acc, sizeof(double) * 16));
    CK(alloc_slots());
    CK(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
    return MIFGPU_OK;
  }

  // Float path: the Dirichlet data of the analytic family is a spatial field
  // times a factor of t, so its faces are evaluated once in double and every
  // boundary fill is one multiplication and one rounding (the working-precision
  // evaluation of exp/sin/cos products cost several ulp of |u| per fill).
  int init_face_tables(mifgpu_ctx *ctx) {
    const int kind = ctx->prm.boundary_kind;
    if (kind == MIFGPU_FIELD_CALLER) return init_caller_tables(ctx);
    if (!std::is_same<T, float>::value || kind == 0 || (g.periodic[0] && g.periodic[1] && g.periodic[2]))
      return MIFGPU_OK;
    long n = 0;
    for (int fn = 0; fn < 2; ++fn)
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) {
          if (g.periodic[d]) continue;
          const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
          for (int sd = 0; sd < 2; ++sd) {
            ftabs.off[fn][c][d][sd] = n;
            n += (long)g.ext(c, a) * g.ext(c, b);
          }
        }
    if (cudaMalloc(&face_tab, sizeof(double) * n) != cudaSuccess)
      return fail(ctx, MIFGPU_ENOMEM, "cudaMalloc of the boundary face tables failed");
    total_bytes += sizeof(double) * n;
    ftabs.tab = face_tab;
    for (int fn = 0; fn < 2; ++fn) launch_face_tables(g, kind, fn, face_tab, ftabs, nullptr);
    CK(cudaDeviceSynchronize());
    return MIFGPU_OK;
  }

  // MIFGPU_FIELD_CALLER: the velocity face tables of the four time slots
  // (slot 0 for mifgpu_apply_bc, slots 1..3 for the stages of the next step),
  // zero until the caller sets them, and the pressure-gradient faces.
  int init_caller_tables(mifgpu_ctx *ctx) {
    long n = 0;
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) {
        if (g.periodic[d]) continue;
        const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
        for (int sd = 0; sd < 2; ++sd) {
          ftabs.off[0][c][d][sd] = n;
          n += (long)g.ext(c, a) * g.ext(c, b);
        }
      }
    const long total = std::max(1L, n) * kCallerSlots;
    if (cudaMalloc(&face_tab, sizeof(double) * total) != cudaSuccess)
      return fail(ctx, MIFGPU_ENOMEM, "cudaMalloc of the caller boundary tables failed");
    total_bytes += sizeof(double) * total;
    CK(cudaMemset(face_tab, 0, sizeof(double) * total));
    ftabs.tab = face_tab;
    ftabs.slot_stride = std::max(1L, n);
    return ensure_grad_faces(ctx);
  }

  static constexpr int kCallerSlots = 4;

  int ensure_grad_faces(mifgpu_ctx *ctx) {
    if (grad_tab) return MIFGPU_OK;
    const long E0 = g.E[0], E1 = g.E[1], E2 = g.E[2];
    const long sz[6] = {E1 * E2, E1 * E2, E0 * E2, E0 * E2, E0 * E1, E0 * E1};
    long n = 0;
    for (int f = 0; f < 6; ++f) {
      gfaces.off[f] = n;
      n += sz[f];
    }
    if (cudaMalloc(&grad_tab, sizeof(double) * n * kCallerSlots) != cudaSuccess)
      return fail(ctx, MIFGPU_ENOMEM, "cudaMalloc of the pressure-gradient face tables failed");
    total_bytes += sizeof(double) * n * kCallerSlots;
    CK(cudaMemset(grad_tab, 0, sizeof(double) * n * kCallerSlots));
    gfaces.tab = grad_tab;
    gfaces.slot_stride = n;
    return MIFGPU_OK;
  }

  // The Dirichlet face planes of host arrays u, v, w (reference layout),
  // packed into slot `slot` of the caller velocity tables.
  int set_boundary_values(mifgpu_ctx *ctx, int slot, const double *const vel[3]) override {
    if (ctx->prm.boundary_kind != MIFGPU_FIELD_CALLER)
      return fail(ctx, MIFGPU_EINVAL, "set_boundary_values needs boundary_kind MIFGPU_FIELD_CALLER");
    pack.assign((size_t)ftabs.slot_stride, 0.0);
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) {
        if (g.periodic[d]) continue;
        const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
        const long ex = g.ext(c, 0), ey = g.ext(c, 1);
        for (int sd = 0; sd < 2; ++sd) {
          double *dst = pack.data() + ftabs.off[0][c][d][sd];
          const long na = g.ext(c, a), nb = g.ext(c, b);
          for (long pb = 0; pb < nb; ++pb)
            for (long pa = 0; pa < na; ++pa) {
              long pt[3];
              pt[a] = pa;
              pt[b] = pb;
              pt[d] = sd ? g.ext(c, d) - 1 : 0;
              dst[pa + na * pb] = vel[c][pt[0] + ex * (pt[1] + ey * pt[2])];
            }
        }
      }
    // a pageable source: the call returns once the data is staged
    CK(cudaMemcpyAsync(face_tab + (size_t)slot * ftabs.slot_stride, pack.data(), sizeof(double) * pack.size(),
                       cudaMemcpyHostToDevice, ctx->stream));
    return MIFGPU_OK;
  }

  int set_gradient_faces(mifgpu_ctx *ctx, int slot, const double *const faces[6]) override {
    if (int rc = ensure_grad_faces(ctx)) return rc;
    for (int f = 0; f < 6; ++f) {
      const long n = (f < 5 ? gfaces.off[f + 1] : gfaces.slot_stride) - gfaces.off[f];
      CK(cudaMemcpyAsync(grad_tab + (size_t)slot * gfaces.slot_stride + gfaces.off[f], faces[f],
                         sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    }
    // pageable sources: each call returns once its data is staged
    return MIFGPU_OK;
  }

  // phi := div(set)/dt + the flux terms of the slot-0 gradient faces, solved
  // (solve_pressure_equation_non_homogeneous_neumann).
  int solve_pressure_nhn(mifgpu_ctx *ctx, int set, double dt) override {
    T *vel[3] = {F.vel(set, 0), F.vel(set, 1), F.vel(set, 2)};
    launch_divergence<T>(g, F.f[kPhi], vel, dt, ctx->stream, &ctx->launches, set_res(set));
    launch_neumann_flux_data<T>(g, F.f[kPhi], gfaces, 0, ctx->stream, &ctx->launches);
    ps.solve(F.f[kPhi], ctx->stream, &ctx->launches);
    CK(cudaGetLastError());
    return MIFGPU_OK;
  }

  // The slot array is allocated once: captured graphs hold its address.
  static constexpr int kMaxSlots = 1024;
  cudaError_t alloc_slots() {
    cudaError_t e = cudaMalloc(&slots, sizeof(double) * kSlotSize * kMaxSlots);
    if (e == cudaSuccess) slots_cap = kMaxSlots;
    return e;
  }

  TimeRef tref() const { return TimeRef{slots, step_ctr}; }

  void remap() {
    F = phys;
    if (parity)
      for (int c = 0; c < 3; ++c) std::swap(F.f[c], F.f[3 + c]);
  }

  // swap_data of velocity and velocity_buffer (src/VelocityTensor.cpp:13-26)
  // as a relabelling: captured graphs exist for both labellings.
  void swap_sets() override {
    parity ^= 1;
    remap();
  }

  void *field_ptr(int id) override { return F.f[id]; }

  Residual residual() const override { return res; }

  // The residual array of field id: the compensated state is velocity set 0
  // between steps, so only its components carry one at the host boundary.
  __nv_bfloat16 *field_res(int id) const { return (res.on() && id < 3) ? res.c[id] : nullptr; }

  // The residuals a sub-step on velocity set `set` uses: set 0's (the state).
  Residual set_res(int set) const { return set == 0 ? res : Residual{}; }

  int ensure_staging(mifgpu_ctx *ctx) {
    const size_t need = (size_t)g.Es[0] * g.Es[1] * g.Es[2];
    if (staging_elems >= need) return MIFGPU_OK;
    cudaFree(staging);
    staging = nullptr;
    if (cudaMalloc(&staging, sizeof(double) * need) != cudaSuccess)
      return fail(ctx, MIFGPU_ENOMEM, "cudaMalloc of the transfer staging buffer failed");
    total_bytes += sizeof(double) * need;
    staging_elems = need;
    return MIFGPU_OK;
  }

  int upload(mifgpu_ctx *ctx, int id, const double *host) override { return upload_fields(ctx, &id, &host, 1); }

  int download(mifgpu_ctx *ctx, int id, double *host) override { return download_fields(ctx, &id, &host, 1); }

  // Slots and copy streams for `count` fields (created on first use).
  int ensure_xfer(mifgpu_ctx *ctx, int count) {
    if (int rc = ensure_staging(ctx)) return rc;
    const size_t need = staging_elems;
    xfer[0] = staging;
    for (int q = 1; q < count; ++q) {
      if (xfer[q] && xfer_elems >= need) continue;
      cudaFree(xfer[q]);
      xfer[q] = nullptr;
      if (cudaMalloc(&xfer[q], sizeof(double) * need) != cudaSuccess)
        return fail(ctx, MIFGPU_ENOMEM, "cudaMalloc of a transfer slot failed");
      total_bytes += sizeof(double) * need;
    }
    if (count > 1) xfer_elems = need;
    for (int c = 0; c < kCopyStreams; ++c) {
      if (!copy_stream[c]) CK(cudaStreamCreateWithFlags(&copy_stream[c], cudaStreamNonBlocking));
      for (auto &row : xfer_ev)
        if (!row[c]) CK(cudaEventCreateWithFlags(&row[c], cudaEventDisableTiming));
    }
    return MIFGPU_OK;
  }

  // Bytes per copy chunk: large enough for full DMA efficiency, small enough
  // that one field spreads over every copy stream.
  static constexpr size_t kChunkElems = size_t(8) << 20;  // 64 MB of doubles

  // Host (reference layout, double) -> fields `ids`: every field's copy is
  // queued at once, in chunks spread over the copy streams, each field's
  // scatter on the context stream after its chunks. The copies start after
  // the context stream's earlier work (a slot may still feed a scatter).
  int upload_fields(mifgpu_ctx *ctx, const int *ids, const double *const *host, int count) {
    if (count < 1 || count > kXferSlots) return MIFGPU_EINVAL;
    if (int rc = ensure_xfer(ctx, count)) return rc;
    cudaEvent_t *start = xfer_ev[kXferSlots];
    CK(cudaEventRecord(start[0], ctx->stream));
    for (int c = 0; c < kCopyStreams; ++c) CK(cudaStreamWaitEvent(copy_stream[c], start[0], 0));
    for (int q = 0; q < count; ++q) {
      int e[3];
      field_extent(g, ids[q], e);
      const size_t n = (size_t)e[0] * e[1] * e[2];
      int c = 0;
      for (size_t off = 0; off < n; off += kChunkElems, c = (c + 1) % kCopyStreams) {
        const size_t len = std::min(kChunkElems, n - off);
        CK(cudaMemcpyAsync(xfer[q] + off, host[q] + off, sizeof(double) * len, cudaMemcpyHostToDevice,
                           copy_stream[c]));
      }
      for (int cs = 0; cs < kCopyStreams; ++cs) {
        CK(cudaEventRecord(xfer_ev[q][cs], copy_stream[cs]));
        CK(cudaStreamWaitEvent(ctx->stream, xfer_ev[q][cs], 0));
      }
      launch_scatter<T>(g, F.f[ids[q]], xfer[q], e[0], e[1], e[2], ctx->stream, &ctx->launches, field_res(ids[q]));
      CK(cudaGetLastError());
    }
    return MIFGPU_OK;
  }

  // Fields `ids` -> host: each field's gather on the context stream, its
  // copy in chunks on the copy streams as soon as the gather is done;
  // returns when every copy has landed.
  int download_fields(mifgpu_ctx *ctx, const int *ids, double *const *host, int count) {
    if (count < 1 || count > kXferSlots) return MIFGPU_EINVAL;
    if (int rc = ensure_xfer(ctx, count)) return rc;
    for (int q = 0; q < count; ++q) {
      int e[3];
      field_extent(g, ids[q], e);
      const size_t n = (size_t)e[0] * e[1] * e[2];
      launch_gather<T>(g, xfer[q], F.f[ids[q]], e[0], e[1], e[2], ctx->stream, &ctx->launches, field_res(ids[q]));
      CK(cudaGetLastError());
      CK(cudaEventRecord(xfer_ev[q][0], ctx->stream));
      for (int c = 0; c < kCopyStreams; ++c) CK(cudaStreamWaitEvent(copy_stream[c], xfer_ev[q][0], 0));
      int c = 0;
      for (size_t off = 0; off < n; off += kChunkElems, c = (c + 1) % kCopyStreams) {
        const size_t len = std::min(kChunkElems, n - off);
        CK(cudaMemcpyAsync(host[q] + off, xfer[q] + off, sizeof(double) * len, cudaMemcpyDeviceToHost,
                           copy_stream[c]));
      }
    }
    for (int c = 0; c < kCopyStreams; ++c) CK(cudaStreamSynchronize(copy_stream[c]));
    CK(cudaStreamSynchronize(ctx->stream));
    return MIFGPU_OK;
  }

  int set_exact(mifgpu_ctx *ctx, int id, double t) override {
    const int comp = id < 9 ? id % 3 : 3;
    launch_set_exact<T>(g, F.f[id], comp, ctx->prm.boundary_kind, t, ctx->stream, &ctx->launches, field_res(id));
    CK(cudaGetLastError());
    return MIFGPU_OK;
  }

  // phi := div(set)/dt (+ Neumann flux) [-> Poisson solve -> periodic refresh]
  void enqueue_pressure(mifgpu_ctx *ctx, cudaStream_t s, int set, double dt, bool nhn, int slot_new, int slot_old,
                        bool solve, long long *cnt, const Residual &r) {
    T *vel[3] = {F.vel(set, 0), F.vel(set, 1), F.vel(set, 2)};
    // The divergence is its own streaming kernel: fused into the x-forward
    // sweep (PoissonSolver::solve's `vel` argument) its loads ran at the line
    // kernel's low occupancy and the pair took 2.5x longer on GB300.
    mark(MIFGPU_PROF_DIVERGENCE, s);
    launch_divergence<T>(g, F.f[kPhi], vel, dt, s, cnt, r);
    if (nhn && ctx->prm.boundary_kind == MIFGPU_FIELD_CALLER)
      launch_neumann_flux_data<T>(g, F.f[kPhi], gfaces, slot_new, s, cnt);
    else if (nhn)
      launch_neumann_flux<T>(g, F.f[kPhi], ctx->prm.boundary_kind, tref(), slot_new, slot_old, s, cnt);
    if (!solve) return;
    std::function<void(int)> mk;
    if (prof) mk = [&](int q) { mark(MIFGPU_PROF_X_FORWARD + q, s); };
    ps.solve(F.f[kPhi], s, cnt, mk);
    mark(MIFGPU_PROF_PERIODIC, s);
    launch_periodic_scalar<T>(g, F.f[kPhi], s, cnt);
  }

  void enqueue_bc(mifgpu_ctx *ctx, cudaStream_t s, int set, int t_slot, long long *cnt, const Residual &r) {
    T *vel[3] = {F.vel(set, 0), F.vel(set, 1), F.vel(set, 2)};
    mark(MIFGPU_PROF_BOUNDARY, s);
    launch_apply_bc<T>(g, vel, ctx->prm.boundary_kind, 0, tref(), t_slot, ftabs, s, cnt, r);
  }

  void enqueue_project(cudaStream_t s, int set, double dt, unsigned tag, long long *cnt, const Residual &r,
                       int *watch = nullptr) {
    T *vel[3] = {F.vel(set, 0), F.vel(set, 1), F.vel(set, 2)};
    mark(MIFGPU_PROF_PROJECT, s);
    launch_project<T>(g, F.f[kP], F.f[kPhi], vel, dt, tref(), tag, s, cnt, r, watch);
  }

  // The kernels of one step of the given variant, in stream order. False
  // if a stage kernel could not be launched (its tensor maps were rejected).
  //
  // Phases (compensated projection steps; every other step is kPhaseFull):
  // in a run of several steps the step's last projection is left to the next
  // step's Y2 stage, which applies it to its ring as the Y3 and U* stages do
  // theirs. The run's first step has no projection to take over (first), the
  // later ones do (rest); the last step of the run ends with the projection
  // kernel (closed), the others do not (open). Sets and pressure after an
  // open step: set 0 and p lack the step's last projection, phi holds it.
  enum { kPhaseFull = 0, kPhaseFirstOpen = 1, kPhaseRestOpen = 2, kPhaseRestClosed = 3 };
  bool enqueue_step(mifgpu_ctx *ctx, cudaStream_t s, int variant, long long *cnt, int phase = kPhaseFull) {
    const double dt = g.dt;
    ForcingTables<T> ft{ftab, ftab_maxE};
    const int kind = ctx->prm.boundary_kind;
    int *const kerr = nonfinite + 1;
    bool ok = true;
    if (variant == kVariantVelocity) {
      StageScalars<T> sc{dt, 4, 1, 0.0};
      const Residual none{};
      ok &= launch_stage<T>(g, F, kVelY2, sc, ft, kind, tref(), s, cnt, none, nullptr, kerr);
      enqueue_bc(ctx, s, 1, 1, cnt, none);
      sc.sin_slot = 6;
      ok &= launch_stage<T>(g, F, kVelY3, sc, ft, kind, tref(), s, cnt, none, nullptr, kerr);
      enqueue_bc(ctx, s, 0, 2, cnt, none);
      sc.sin_slot = 8;
      ok &= launch_stage<T>(g, F, kVelUStar, sc, ft, kind, tref(), s, cnt, none, nullptr, kerr);
      enqueue_bc(ctx, s, 1, 3, cnt, none);
      return ok;  // the final swap of sets 0 and 1 is done on the host side
    }
    const bool nhn = variant == kVariantNhn;
    const double dts[3] = {64.0 / 120.0 * dt, 16.0 / 120.0 * dt, 40.0 / 120.0 * dt};
    const StageKind kinds[3] = {kStageY2, kStageY3, kStageUStar};
    const int out_set[3] = {1, 2, 0};
    const int sin_slot[3] = {4, 6, 8};
    // In the compensated state the Y3 and U* stage kernels apply the
    // projection before them (StageProj): the projected sets 1 and 2 are read
    // by those stages only, so they are never stored. The pressure goes
    // p -> p_alt (Y3) -> p (U*), and the last projection is a kernel of its own
    // (or, in the rest phases, p -> p_alt (Y2) -> p_alt2 (Y3) -> p (U*)).
    const bool fused = res.on() && p_alt;
    const bool rest = fused && (phase == kPhaseRestOpen || phase == kPhaseRestClosed);
    const bool closed = !fused || phase == kPhaseFull || phase == kPhaseRestClosed;
    T *const pbuf[4] = {F.f[kP], p_alt, rest ? p_alt2 : F.f[kP], F.f[kP]};  // p before stage st, after U*
    for (int st = 0; st < 3; ++st) {
      StageScalars<T> sc{dt, sin_slot[st], ctx->prm.forcing, ctx->prm.forcing_amplitude};
      StageProj pj{};
      const bool proj = fused && (st > 0 || rest);
      if constexpr (std::is_same<T, float>::value) {
        // stage st applies the projection of stage st - 1 (the previous
        // step's U* for the Y2 stage)
        const int prev = st == 0 ? 2 : st - 1;
        pj.phi = F.f[kPhi];
        pj.p_in = rest ? pbuf[st] : (st == 1 ? F.f[kP] : p_alt);
        pj.p_out = rest ? pbuf[st + 1] : (st == 1 ? p_alt : F.f[kP]);
        pj.dt = float(dts[prev]);
        pj.tag = 16u + prev;
      }
      // in the compensated state every stage's output set carries the residuals
      mark(MIFGPU_PROF_STAGE, s);
      ok &= launch_stage<T>(g, F, kinds[st], sc, ft, kind, tref(), s, cnt, res, proj ? &pj : nullptr, kerr);
      enqueue_bc(ctx, s, out_set[st], 1 + st, cnt, res);
      enqueue_pressure(ctx, s, out_set[st], dts[st], nhn, 1 + st, st, true, cnt, res);
      // the last projection of the step watches phi for NaN / Inf
      if (!fused || (st == 2 && closed))
        enqueue_project(s, out_set[st], dts[st], 16u + st, cnt, res, st == 2 ? nonfinite : nullptr);
    }
    return ok;
  }

  int ensure_graph(mifgpu_ctx *ctx, int variant, int phase = kPhaseFull) {
    if (graph[variant][parity][phase]) return MIFGPU_OK;
    cudaGraph_t gr = nullptr;
    CK(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal));
    long long cnt = 0;
    const bool launched = enqueue_step(ctx, cap_stream, variant, &cnt, phase);
    advance_step_kernel<<<1, 1, 0, cap_stream>>>(step_ctr);
    ++cnt;
    cudaError_t e = cudaStreamEndCapture(cap_stream, &gr);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "stream capture of the step");
    if (!launched) {
      cudaGraphDestroy(gr);
      return fail(ctx, MIFGPU_ECUDA, "cuTensorMapEncodeTiled rejected a stage kernel's tile map");
    }
    e = cudaGraphInstantiate(&graph[variant][parity][phase], gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
    graph_launches[variant][parity][phase] = cnt;
    return MIFGPU_OK;
  }

  // `nsteps` replays of the step graph of `variant`. The velocity-only step
  // ends with the swap of sets 0 and 1 (src/TimestepVelocity.cpp:89), a
  // relabelling: its replays alternate the graphs of the two labellings.
  int step(mifgpu_ctx *ctx, int variant, const double *host_slots, int nsteps) override {
    const bool swap = variant == kVariantVelocity;
    // the compensated projection steps of a run of several steps hand each
    // step's last projection to the next step (enqueue_step's phases)
    const bool chain = res.on() && p_alt && !swap && nsteps > 1;
    auto phase_of = [&](int n) {
      return !chain ? kPhaseFull : n == 0 ? kPhaseFirstOpen : n == nsteps - 1 ? kPhaseRestClosed : kPhaseRestOpen;
    };
    if (chain) {
      for (int ph : {kPhaseFirstOpen, kPhaseRestOpen, kPhaseRestClosed})
        if (int rc = ensure_graph(ctx, variant, ph)) return rc;
    } else if (int rc = ensure_graph(ctx, variant)) {
      return rc;
    }
    if (swap && nsteps > 1) {
      swap_sets();
      const int rc = ensure_graph(ctx, variant);
      swap_sets();
      if (rc) return rc;
    }
    CK(cudaMemsetAsync(nonfinite, 0, 2 * sizeof(int), ctx->stream));
    for (int n0 = 0; n0 < nsteps; n0 += slots_cap) {
      const int chunk = std::min(slots_cap, nsteps - n0);
      CK(cudaMemcpyAsync(slots, host_slots + (size_t)kSlotSize * n0, sizeof(double) * kSlotSize * chunk,
                         cudaMemcpyHostToDevice, ctx->stream));
      CK(cudaMemsetAsync(step_ctr, 0, sizeof(int), ctx->stream));
      for (int n = 0; n < chunk; ++n) {
        const int ph = phase_of(n0 + n);
        CK(cudaGraphLaunch(graph[variant][parity][ph], ctx->stream));
        ctx->launches += graph_launches[variant][parity][ph];
        if (swap) swap_sets();
      }
    }
    // The host copy of the slots may be a temporary: wait until it was consumed.
    int bad[2] = {0, 0};
    CK(cudaMemcpyAsync(bad, nonfinite, sizeof(bad), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (bad[1]) return fail(ctx, MIFGPU_ECUDA, "a stage or line kernel gave up waiting for a TMA tile load");
    if (bad[0])
      return fail(ctx, MIFGPU_ENONFINITE,
                  "a projection step produced a NaN or Inf pressure increment (the velocity or pressure is no longer "
                  "finite)");
    return MIFGPU_OK;
  }

  int profile_step(mifgpu_ctx *ctx, double t_n, int reps, double *ms) override {
    double sl[kSlotSize];
    projection_slot(t_n, g.dt, ctx->prm.boundary_kind, g.Re, sl);
    CK(cudaMemcpyAsync(slots, sl, sizeof(sl), cudaMemcpyHostToDevice, ctx->stream));
    for (int c = 0; c < MIFGPU_PROF_CLASSES; ++c) ms[c] = 0.0;
    // In the compensated state the step timed is the one a run repeats (its
    // Y2 stage applies the previous step's last projection, and it has no
    // projection kernel): one untimed step before it leaves a projection to
    // apply, one untimed step after applies the last one.
    const bool chain = res.on() && p_alt;
    auto untimed = [&](int phase) {
      CK(cudaMemsetAsync(step_ctr, 0, sizeof(int), ctx->stream));
      if (!enqueue_step(ctx, ctx->stream, kVariantProjection, &ctx->launches, phase))
        return fail(ctx, MIFGPU_ECUDA, "cuTensorMapEncodeTiled rejected a stage kernel's tile map");
      CK(cudaStreamSynchronize(ctx->stream));
      return MIFGPU_OK;
    };
    CK(cudaMemsetAsync(nonfinite, 0, 2 * sizeof(int), ctx->stream));
    if (chain)
      if (int rc = untimed(kPhaseFirstOpen)) return rc;
    for (int r = 0; r < reps; ++r) {
      std::vector<std::pair<int, cudaEvent_t>> marks;
      prof = &marks;
      CK(cudaMemsetAsync(step_ctr, 0, sizeof(int), ctx->stream));
      const bool launched =
          enqueue_step(ctx, ctx->stream, kVariantProjection, &ctx->launches, chain ? kPhaseRestOpen : kPhaseFull);
      mark(-1, ctx->stream);
      prof = nullptr;
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (!launched) {
        for (auto &m : marks) cudaEventDestroy(m.second);
        return fail(ctx, MIFGPU_ECUDA, "cuTensorMapEncodeTiled rejected a stage kernel's tile map");
      }
      for (size_t q = 0; q + 1 < marks.size(); ++q) {
        float t = 0.f;
        cudaEventElapsedTime(&t, marks[q].second, marks[q + 1].second);
        ms[marks[q].first] += t / reps;
      }
      for (auto &m : marks) cudaEventDestroy(m.second);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "profiled step");
    }
    if (chain)
      if (int rc = untimed(kPhaseRestClosed)) return rc;
    int flags[2] = {0, 0};
    CK(cudaMemcpy(flags, nonfinite, sizeof(flags), cudaMemcpyDeviceToHost));
    if (flags[1]) return fail(ctx, MIFGPU_ECUDA, "a stage or line kernel gave up waiting for a TMA tile load");
    return MIFGPU_OK;
  }

  int write_single_slot(mifgpu_ctx *ctx, double t) {
    double s[kSlotSize];
    projection_slot(t, g.dt, ctx->prm.boundary_kind, g.Re, s);
    s[1] = s[2] = s[3] = t;  // sub-step calls use their own time in every slot
    slot_factors(s, ctx->prm.boundary_kind, g.Re);
    CK(cudaMemcpyAsync(slots, s, sizeof(s), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(step_ctr, 0, sizeof(int), ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return MIFGPU_OK;
  }

  int apply_bc(mifgpu_ctx *ctx, int set, double t) override {
    if (int rc = write_single_slot(ctx, t)) return rc;
    enqueue_bc(ctx, ctx->stream, set, 0, &ctx->launches, set_res(set));
    CK(cudaGetLastError());
    return MIFGPU_OK;
  }

  int solve_pressure(mifgpu_ctx *ctx, int set, double dt, bool solve) override {
    enqueue_pressure(ctx, ctx->stream, set, dt, false, 0, 0, solve, &ctx->launches, set_res(set));
    CK(cudaGetLastError());
    return MIFGPU_OK;
  }

  int project(mifgpu_ctx *ctx, int set, double dt) override {
    // the kernel reads time slot 0 (its rounding draw): point the step
    // counter at a written slot
    if (int rc = write_single_slot(ctx, 0.0)) return rc;
    enqueue_project(ctx->stream, set, dt, 15u, &ctx->launches, set_res(set));
    CK(cudaGetLastError());
    return MIFGPU_OK;
  }

  int adjust_pressure(mifgpu_ctx *ctx, double t) override {
    CK(cudaMemsetAsync(acc, 0, sizeof(double) * 4, ctx->stream));
    launch_pressure_mean_diff<T>(g, F.f[kP], ctx->prm.boundary_kind, t, acc, ctx->stream, &ctx->launches);
    launch_add_scalar<T>(g, F.f[kP], acc, ctx->stream, &ctx->launches);
    CK(cudaGetLastError());
    return MIFGPU_OK;
  }

  int error_norms(mifgpu_ctx *ctx, double t, double out[9]) override {
    const int kind = ctx->prm.boundary_kind;
    if (!grad_block) {
      if (cudaMalloc(&grad_block, sizeof(T) * field_elems * 3) != cudaSuccess)
        return fail(ctx, MIFGPU_ENOMEM, "cudaMalloc of the gradient scratch failed");
      total_bytes += sizeof(T) * field_elems * 3;
      CK(cudaMemset(grad_block, 0, sizeof(T) * field_elems * 3));
    }
    T *gv[3] = {grad_block, grad_block + field_elems, grad_block + 2 * field_elems};
    T *vel[3] = {F.vel(0, 0), F.vel(0, 1), F.vel(0, 2)};
    CK(cudaMemsetAsync(acc, 0, sizeof(double) * 9, ctx->stream));
    launch_velocity_errors<T>(g, vel, kind, 0, t, acc, ctx->stream, &ctx->launches, res);
    launch_pressure_errors<T>(g, F.f[kP], kind, t, acc + 3, ctx->stream, &ctx->launches);
    launch_pressure_gradient<T>(g, gv, F.f[kP], ctx->stream, &ctx->launches);
    if (int rc = write_single_slot(ctx, t)) return rc;
    launch_apply_bc<T>(g, gv, kind, 1, tref(), 0, ftabs, ctx->stream, &ctx->launches);
    launch_velocity_errors<T>(g, gv, kind, 1, t, acc + 6, ctx->stream, &ctx->launches);
    double h[9];
    CK(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const double vol = g.h[0] * g.h[1] * g.h[2];
    for (int b = 0; b < 3; ++b) {
      const double *a = h + 3 * b;
      out[3 * b + 0] = a[0] * vol;  // sum of |e| (of the error vector for velocity and gradient)
      out[3 * b + 1] = std::sqrt(a[1] * vol);
      out[3 * b + 2] = a[2];
    }
    return MIFGPU_OK;
  }

  // ---- reverse mode ----

  T *adj_field(int q) const { return adj_block + (size_t)q * field_elems; }
  enum { kLX = 0, kMU = 3, kPEND = 6, kRHO = 9, kLP = 10, kAdjFields = 11 };

  int ensure_fields(mifgpu_ctx *ctx, T *&buf, size_t &have, size_t need, const char *what) {
    if (have >= need) return MIFGPU_OK;
    cudaFree(buf);
    buf = nullptr;
    total_bytes -= sizeof(T) * field_elems * have;
    have = 0;
    if (cudaMalloc(&buf, sizeof(T) * field_elems * need) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, MIFGPU_ENOMEM, std::string("cudaMalloc of the ") + what + " failed");
    }
    have = need;
    total_bytes += sizeof(T) * field_elems * need;
    return MIFGPU_OK;
  }

  cudaError_t copy_fields(T *dst, const T *src, int n, cudaStream_t s) {
    return cudaMemcpyAsync(dst, src, sizeof(T) * field_elems * n, cudaMemcpyDeviceToDevice, s);
  }

  // Adjoint of one projection step (src/Timestep.cpp:97-141) given the
  // adjoint of its output in lx (velocity set 0) and lp (pressure), and the
  // sets the three stage right-hand sides were evaluated at: V[0] = u_n,
  // V[1] = set 1 and V[2] = set 2 after the step. Leaves the adjoint of the
  // step's input in lx and lp and adds d loss / d alpha into *dalpha.
  // False if a tensor map of the adjoint stencil was rejected (its launch
  // and the rest of the step are then left out).
  bool reverse_step(mifgpu_ctx *ctx, cudaStream_t s, const T *const V[3][3], double *dalpha, long long *cnt) {
    using Ops = AdjointOps<T>;
    const double dt = g.dt;
    T *lx[3] = {adj_field(kLX), adj_field(kLX + 1), adj_field(kLX + 2)};
    T *mu[3] = {adj_field(kMU), adj_field(kMU + 1), adj_field(kMU + 2)};
    T *pend[3] = {adj_field(kPEND), adj_field(kPEND + 1), adj_field(kPEND + 2)};
    T *rho = adj_field(kRHO), *lp = adj_field(kLP);
    // Stage k: projection step dt_k, weight of its own R, weight of grad p,
    // and the weight of the previous stage's R that its update carries.
    const double dts[3] = {64.0 / 120.0 * dt, 16.0 / 120.0 * dt, 40.0 / 120.0 * dt};
    const double a_own[3] = {64.0 / 120.0 * dt, 50.0 / 120.0 * dt, 90.0 / 120.0 * dt};
    const double b_p[3] = {64.0 / 120.0 * dt, 16.0 / 120.0 * dt, 40.0 / 120.0 * dt};
    const double a_prev[3] = {0.0, -34.0 / 120.0 * dt, -50.0 / 120.0 * dt};
    const bool tg = ctx->prm.forcing == MIFGPU_FORCING_TAYLOR_GREEN;
    for (int st = 2; st >= 0; --st) {
      // phi = P M D X / dt_k, p += phi, X -= dt_k G phi on the interior
      Ops::grad_adjoint(g, rho, lp, lx, -dts[st], true, s, cnt);
      Ops::periodic_scalar_adjoint(g, rho, s, cnt);
      ps.solve(rho, s, cnt);
      Ops::div_adjoint(g, lx, lx, rho, 1.0 / dts[st], s, cnt);
      // boundary fill of the stage's output set
      Ops::bc_adjoint(g, lx, s, cnt);
      // X = prev + a_own R(prev) + a_prev R_prev - b_p G p on the interior
      Ops::grad_adjoint(g, lp, lp, lx, -b_p[st], false, s, cnt);
      Ops::split(g, mu, pend, lx, a_own[st], st < 2 ? 1.0 : 0.0, a_prev[st], st > 0, tg ? ftab : nullptr, ftab_maxE,
                 red_part, dalpha, s, cnt);
      if (!Ops::rhs_adjoint(g, lx, mu, V[st], s, cnt, nonfinite + 1)) return false;
    }
    return true;
  }

  // The reverse step of snapshot slot m as a graph, captured on first use.
  int ensure_rev_graph(mifgpu_ctx *ctx, int m, const T *const V[3][3]) {
    if ((int)rev_graph.size() <= m) rev_graph.resize(m + 1, nullptr);
    if (rev_graph[m]) return MIFGPU_OK;
    cudaGraph_t gr = nullptr;
    CK(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal));
    long long n = 0;
    const bool maps_ok = reverse_step(ctx, cap_stream, V, acc + 1, &n);
    cudaError_t e = cudaStreamEndCapture(cap_stream, &gr);
    if (e == cudaSuccess && !maps_ok) {
      cudaGraphDestroy(gr);
      return fail(ctx, MIFGPU_ECUDA, "a TMA tensor map of the adjoint stencil was rejected");
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "stream capture of the reverse step");
    e = cudaGraphInstantiate(&rev_graph[m], gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate (reverse step)");
    rev_graph_launches = n;
    return MIFGPU_OK;
  }

  void drop_rev_graphs() {
    for (auto &gx : rev_graph)
      if (gx) cudaGraphExecDestroy(gx);
    rev_graph.clear();
  }

  int gradient(mifgpu_ctx *ctx, const GradRequest &req) override {
    if (res.on())
      return fail(ctx, MIFGPU_ENOTSUP, "the reverse mode runs in MIFGPU_FP64 or MIFGPU_MIXED, not on a compensated state");
    const int N = req.nsteps;
    const int C = std::max(1, std::min(req.every, N));
    if (C > slots_cap) return fail(ctx, MIFGPU_EINVAL, "checkpoint interval above 1024 steps");
    const int nseg = (N + C - 1) / C;
    if (!adj_block) {
      size_t have_adj = 0;
      if (int rc = ensure_fields(ctx, adj_block, have_adj, kAdjFields, "adjoint fields")) return rc;
      // mu must read 0 off the interior, padding included (the split kernel
      // never writes the padding)
      CK(cudaMemset(adj_block, 0, sizeof(T) * field_elems * kAdjFields));
      const long nb = AdjointOps<T>::box_blocks(g);
      if (cudaMalloc(&red_part, sizeof(double) * nb) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, MIFGPU_ENOMEM, "cudaMalloc of the adjoint partial sums failed");
      }
      total_bytes += sizeof(double) * nb;
      CK(AdjointOps<T>::prepare());
    }
    if (int rc = ensure_fields(ctx, ckpt_block, ckpt_fields, (size_t)4 * (nseg + 1), "checkpoints")) return rc;
    // Two snapshot buffers of 9 C fields, so that one segment's recompute
    // can run beside the previous segment's reverse sweep; one if two do not
    // fit (then the two alternate on the GPU).
    T *const snap_before = snap_block;
    if (snap_fields < (size_t)18 * C && ensure_fields(ctx, snap_block, snap_fields, (size_t)18 * C, "segment snapshots")) {
      cudaGetLastError();
      if (int rc = ensure_fields(ctx, snap_block, snap_fields, (size_t)9 * C, "segment snapshots")) return rc;
    }
    if (snap_block != snap_before) drop_rev_graphs();
    const int nbuf = snap_fields >= (size_t)18 * C ? 2 : 1;
    if (!rec_stream) CK(cudaStreamCreateWithFlags(&rec_stream, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
      if (!ev_rec[b]) CK(cudaEventCreateWithFlags(&ev_rec[b], cudaEventDisableTiming));
      if (!ev_rev[b]) CK(cudaEventCreateWithFlags(&ev_rev[b], cudaEventDisableTiming));
    }
    if (int rc = ensure_graph(ctx, kVariantProjection)) return rc;
    cudaStream_t s = ctx->stream, r = rec_stream;
    CK(cudaMemsetAsync(nonfinite, 0, 2 * sizeof(int), s));
    long long *cnt = &ctx->launches;
    std::vector<double> sl((size_t)kSlotSize * N);
    for (int n = 0; n < N; ++n)
      projection_slot(req.t0 + n * g.dt, g.dt, ctx->prm.boundary_kind, g.Re, sl.data() + (size_t)kSlotSize * n);
    T *set0 = F.vel(0, 0), *set1 = F.vel(1, 0), *set2 = F.vel(2, 0), *p = F.f[kP];
    auto ck = [&](int seg) { return ckpt_block + (size_t)4 * seg * field_elems; };
    // snapshot slot q = b C + m: step m of a segment in buffer b
    auto sn = [&](int q) { return snap_block + (size_t)9 * q * field_elems; };
    // timing events: forward start / end, backward end, and per segment the
    // start and end of its reverse sweep on the reverse stream
    std::vector<cudaEvent_t> evs;
    auto stamp = [&](cudaStream_t st) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      cudaEventRecord(e, st);
      evs.push_back(e);
      return e;
    };
    auto cleanup = [&]() {
      for (auto &e : evs) cudaEventDestroy(e);
    };
    // the steps of segment seg from its checkpointed start on stream st; with
    // snapshots into buffer b, the three sets each stage's right-hand side
    // is evaluated at
    auto run_seg = [&](int seg, int b, cudaStream_t st) -> cudaError_t {
      const int n0 = seg * C, len = std::min(C, N - n0);
      cudaError_t e = cudaMemcpyAsync(slots, sl.data() + (size_t)kSlotSize * n0, sizeof(double) * kSlotSize * len,
                                      cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaMemsetAsync(step_ctr, 0, sizeof(int), st);
      for (int m = 0; m < len && e == cudaSuccess; ++m) {
        T *snap = b >= 0 ? sn(b * C + m) : nullptr;
        if (snap) e = copy_fields(snap, set0, 3, st);
        if (e == cudaSuccess) e = cudaGraphLaunch(graph[kVariantProjection][parity][kPhaseFull], st);
        *cnt += graph_launches[kVariantProjection][parity][kPhaseFull];
        if (snap && e == cudaSuccess) e = copy_fields(snap + 3 * field_elems, set1, 3, st);
        if (snap && e == cudaSuccess) e = copy_fields(snap + 6 * field_elems, set2, 3, st);
      }
      return e;
    };
    // forward pass, one checkpoint per segment start and one of the final state
    cudaEvent_t t_fwd0 = stamp(s);
    for (int seg = 0; seg < nseg; ++seg) {
      cudaError_t e = copy_fields(ck(seg), set0, 3, s);
      if (e == cudaSuccess) e = copy_fields(ck(seg) + 3 * field_elems, p, 1, s);
      if (e == cudaSuccess) e = run_seg(seg, -1, s);
      if (e != cudaSuccess) return cleanup(), cuda_fail(ctx, e, "forward pass");
    }
    CK(copy_fields(ck(nseg), set0, 3, s));
    CK(copy_fields(ck(nseg) + 3 * field_elems, p, 1, s));
    cudaEvent_t t_fwd1 = stamp(s);
    // seed the adjoint of the final state
    T *lx[3] = {adj_field(kLX), adj_field(kLX + 1), adj_field(kLX + 2)};
    CK(cudaMemsetAsync(acc, 0, sizeof(double) * 2, s));
    if (req.box) {
      const T *u[3] = {set0, set0 + field_elems, set0 + 2 * field_elems};
      AdjointOps<T>::ke_seed(g, u, lx, req.box, red_part, acc, s, cnt);
      CK(cudaMemsetAsync(adj_field(kLP), 0, sizeof(T) * field_elems, s));
    } else {
      for (int q = 0; q < 3; ++q) CK(cudaMemsetAsync(lx[q], 0, sizeof(T) * field_elems, s));
      CK(cudaMemsetAsync(adj_field(kLP), 0, sizeof(T) * field_elems, s));
      if (int rc = ensure_staging(ctx)) return cleanup(), rc;
      const int ids[4] = {0, 1, 2, kP};
      T *dst[4] = {lx[0], lx[1], lx[2], adj_field(kLP)};
      for (int q = 0; q < 4; ++q) {
        if (!req.seed[q]) continue;
        int e3[3];
        field_extent(g, ids[q], e3);
        const size_t n = (size_t)e3[0] * e3[1] * e3[2];
        CK(cudaMemcpyAsync(staging, req.seed[q], sizeof(double) * n, cudaMemcpyHostToDevice, s));
        launch_scatter<T>(g, dst[q], staging, e3[0], e3[1], e3[2], s, cnt);
      }
    }
    // the recompute stream starts once the seed has read the final state
    CK(cudaStreamWaitEvent(r, stamp(s), 0));
    // backward: per segment, recompute it with snapshots (stream r), then
    // reverse its steps (stream s). A buffer passes from a reverse sweep to
    // the next recompute into it through ev_rev, and back through ev_rec.
    auto recompute = [&](int seg) -> int {
      const int b = seg % nbuf;
      CK(cudaStreamWaitEvent(r, ev_rev[b], 0));
      cudaError_t e = copy_fields(set0, ck(seg), 3, r);
      if (e == cudaSuccess) e = copy_fields(p, ck(seg) + 3 * field_elems, 1, r);
      if (e == cudaSuccess) e = run_seg(seg, b, r);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "segment recompute");
      CK(cudaEventRecord(ev_rec[b], r));
      return MIFGPU_OK;
    };
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> sweeps;
    auto reverse = [&](int seg) -> int {
      const int b = seg % nbuf, len = std::min(C, N - seg * C);
      CK(cudaStreamWaitEvent(s, ev_rec[b], 0));
      cudaEvent_t e0 = stamp(s);
      for (int m = len - 1; m >= 0; --m) {
        const int q = b * C + m;
        const T *V[3][3];
        for (int st = 0; st < 3; ++st)
          for (int c = 0; c < 3; ++c) V[st][c] = sn(q) + (size_t)(3 * st + c) * field_elems;
        if (int rc = ensure_rev_graph(ctx, q, V)) return rc;
        CK(cudaGraphLaunch(rev_graph[q], s));
        *cnt += rev_graph_launches;
      }
      sweeps.push_back({e0, stamp(s)});
      CK(cudaEventRecord(ev_rev[b], s));
      return MIFGPU_OK;
    };
    if (int rc = recompute(nseg - 1)) return cleanup(), rc;
    for (int seg = nseg - 1; seg >= 0; --seg) {
      // with two buffers the next segment's recompute runs beside this sweep
      if (nbuf == 2 && seg > 0)
        if (int rc = recompute(seg - 1)) return cleanup(), rc;
      if (int rc = reverse(seg)) return cleanup(), rc;
      if (nbuf == 1 && seg > 0)
        if (int rc = recompute(seg - 1)) return cleanup(), rc;
    }
    // the reverse stream takes over the forward fields again
    cudaEvent_t r_done = stamp(r);
    CK(cudaStreamWaitEvent(s, r_done, 0));
    cudaEvent_t t_bwd1 = stamp(s);
    // leave the context at the final state
    CK(copy_fields(set0, ck(nseg), 3, s));
    CK(copy_fields(p, ck(nseg) + 3 * field_elems, 1, s));
    double h[2];
    int flags[2] = {0, 0};
    CK(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(flags, nonfinite, sizeof(flags), cudaMemcpyDeviceToHost, s));
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cleanup(), cuda_fail(ctx, e, "gradient");
    if (flags[1])
      return cleanup(), fail(ctx, MIFGPU_ECUDA, "a stage, line or adjoint kernel gave up waiting for a TMA tile load");
    if (req.loss) *req.loss = h[0];
    if (req.dalpha) *req.dalpha = h[1];
    if (req.ms) {
      float t = 0.f;
      cudaEventElapsedTime(&t, t_fwd0, t_fwd1);
      req.ms[0] = t;
      cudaEventElapsedTime(&t, t_fwd1, t_bwd1);
      req.ms[1] = t;
      req.ms[2] = 0.0;
      for (auto &sw : sweeps) {
        cudaEventElapsedTime(&t, sw.first, sw.second);
        req.ms[2] += t;
      }
    }
    cleanup();
    return MIFGPU_OK;
  }

  int download_adjoint(mifgpu_ctx *ctx, int id, double *host) override {
    if (!adj_block) return fail(ctx, MIFGPU_EINVAL, "no adjoint has been computed on this context");
    int e[3];
    field_extent(g, id, e);
    if (int rc = ensure_staging(ctx)) return rc;
    const size_t n = (size_t)e[0] * e[1] * e[2];
    const T *src = id == kP ? adj_field(kLP) : adj_field(kLX + id);
    launch_gather<T>(g, staging, src, e[0], e[1], e[2], ctx->stream, &ctx->launches);
    CK(cudaMemcpyAsync(host, staging, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return MIFGPU_OK;
  }

  int fetch_box(mifgpu_ctx *ctx, int id, const int lo[3], const int n[3], double *out) override {
    if (int rc = ensure_staging(ctx)) return rc;
    const T *src = id == kP ? F.f[kP] : F.vel(0, id);
    const dim3 grid((unsigned)((n[0] + 31) / 32), (unsigned)((n[1] + 7) / 8), (unsigned)n[2]);
    box_gather_kernel<T><<<grid, dim3(32, 8), 0, ctx->stream>>>(g, staging, src, lo[0], lo[1], lo[2], n[0], n[1]);
    ++ctx->launches;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, staging, sizeof(double) * (size_t)n[0] * n[1] * n[2], cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return MIFGPU_OK;
  }

  // Captured graphs hold the stage scalars: drop them when one changes.
  void drop_graphs() override {
    drop_rev_graphs();
    for (auto &gv : graph)
      for (auto &gp : gv)
        for (auto &gx : gp)
          if (gx) {
            cudaGraphExecDestroy(gx);
            gx = nullptr;
          }
  }

  size_t bytes() const override { return total_bytes; }
};

bool valid_field(int id) { return id >= 0 && id < kNumFields; }

}  // namespace

extern "C" {

int mifgpu_create(const mifgpu_params *p, mifgpu_ctx **out) {
  if (!p || !out) return MIFGPU_EINVAL;
  *out = nullptr;
  auto ctx = std::make_unique<mifgpu_ctx>();
  ctx->prm = *p;
  if (p->precision != MIFGPU_FP64 && p->precision != MIFGPU_MIXED && p->precision != MIFGPU_MIXED_COMPENSATED)
    return MIFGPU_EINVAL;
  if (p->boundary_kind < 0 || p->boundary_kind > 3 || p->forcing < 0 || p->forcing > 3) return MIFGPU_EINVAL;
  if (!(p->Re > 0) || !(p->dt > 0)) return MIFGPU_EINVAL;
  Geometry &g = ctx->g;
  for (int d = 0; d < 3; ++d) {
    const int per = p->periodic[d] != 0;
    if (p->n_global[d] < 3 || p->n_global[d] > (1 << 20) || !(p->size[d] > 0)) return MIFGPU_EINVAL;
    g.n_global[d] = (int)p->n_global[d];
    g.periodic[d] = per;
    g.h[d] = p->size[d] / (double)(p->n_global[d] - 1);
    g.oh[d] = 1 / g.h[d];
    g.o2h[d] = 1 / (2 * g.h[d]);
    g.o8h[d] = 1 / (8 * g.h[d]);
    g.oh2Re[d] = 1 / (p->Re * g.h[d] * g.h[d]);
    g.h_2[d] = g.h[d] / 2;
    g.origin[d] = p->origin[d];
    g.E[d] = per ? g.n_global[d] + 1 : g.n_global[d];
    g.base[d] = per ? -1 : 0;
    g.np[d] = g.n_global[d] - per;
    g.own_lo[d] = per;
  }
  // One rank: the y and z staggered extents always gain a point, x only on a
  // Dirichlet axis (src/Constants.cpp:86-88).
  g.Es[0] = g.periodic[0] ? g.E[0] : g.E[0] + 1;
  g.Es[1] = g.E[1] + 1;
  g.Es[2] = g.E[2] + 1;
  // CUDA grids hold at most 65535 blocks along y and z. The box kernels give
  // every z plane of a staggered field its own grid-z block, the stencil
  // kernels tile y in rows of 4, and the face kernels tile the longest
  // extent in rows of 8. A longer axis is refused here, before any device
  // work, instead of failing at its first launch.
  constexpr long kGridYZ = 65535;
  if (g.Es[2] > kGridYZ || g.Es[1] > 4 * kGridYZ || std::max({g.Es[0], g.Es[1], g.Es[2]}) > 8 * kGridYZ)
    return MIFGPU_EINVAL;
  g.PX = ((long)std::max(g.Es[0], g.E[0]) + 7) / 8 * 8;
  g.PY = g.Es[1];
  g.PZ = g.Es[2];
  g.Re = p->Re;
  g.dt = p->dt;
  if (cudaGetDevice(&ctx->device) != cudaSuccess) return fail(nullptr, MIFGPU_ECUDA, "no CUDA device");
  if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess) return MIFGPU_ECUDA;
  ctx->stream = ctx->own_stream;
  if (p->precision == MIFGPU_FP64)
    ctx->impl = std::make_unique<Impl<double>>();
  else
    ctx->impl = std::make_unique<Impl<float>>();
  const int rc = ctx->impl->init(ctx.get());
  if (rc != MIFGPU_OK) {
    // keep the context so the caller can read the message
    *out = ctx.release();
    return rc;
  }
  *out = ctx.release();
  return MIFGPU_OK;
}

int mifgpu_destroy(mifgpu_ctx *ctx) {
  if (!ctx) return MIFGPU_EINVAL;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->impl.reset();
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return MIFGPU_OK;
}

int mifgpu_set_stream(mifgpu_ctx *ctx, void *stream) {
  if (!ctx) return MIFGPU_EINVAL;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return MIFGPU_OK;
}

int mifgpu_synchronize(mifgpu_ctx *ctx) {
  if (!ctx) return MIFGPU_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  return MIFGPU_OK;
}

const char *mifgpu_last_error(const mifgpu_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int mifgpu_field_extent(const mifgpu_ctx *ctx, int field, long out[3]) {
  if (!ctx || !out || !valid_field(field)) return MIFGPU_EINVAL;
  int e[3];
  field_extent(ctx->g, field, e);
  for (int d = 0; d < 3; ++d) out[d] = e[d];
  return MIFGPU_OK;
}

int mifgpu_upload(mifgpu_ctx *ctx, int field, const double *host) {
  if (!ctx || !host || !valid_field(field)) return MIFGPU_EINVAL;
  return ctx->impl->upload(ctx, field, host);
}

int mifgpu_download(mifgpu_ctx *ctx, int field, double *host) {
  if (!ctx || !host || !valid_field(field)) return MIFGPU_EINVAL;
  return ctx->impl->download(ctx, field, host);
}

namespace {
// Entry points that evaluate the analytic family have nothing to evaluate
// when the caller supplies the boundary data.
int needs_family(mifgpu_ctx *ctx, const char *what) {
  if (ctx->prm.boundary_kind != MIFGPU_FIELD_CALLER) return MIFGPU_OK;
  return fail(ctx, MIFGPU_ENOTSUP,
              std::string(what) + " evaluates the analytic family; boundary_kind MIFGPU_FIELD_CALLER has none");
}
}  // namespace

int mifgpu_set_exact_velocity(mifgpu_ctx *ctx, int set, double t) {
  if (!ctx || set < 0 || set > 2) return MIFGPU_EINVAL;
  if (int rc = needs_family(ctx, "set_exact_velocity")) return rc;
  for (int c = 0; c < 3; ++c)
    if (int rc = ctx->impl->set_exact(ctx, set * 3 + c, t)) return rc;
  return MIFGPU_OK;
}

int mifgpu_set_exact_pressure(mifgpu_ctx *ctx, double t) {
  if (!ctx) return MIFGPU_EINVAL;
  if (int rc = needs_family(ctx, "set_exact_pressure")) return rc;
  return ctx->impl->set_exact(ctx, kP, t);
}

int mifgpu_timestep(mifgpu_ctx *ctx, double t_n) {
  if (!ctx) return MIFGPU_EINVAL;
  double s[kSlotSize];
  projection_slot(t_n, ctx->g.dt, ctx->prm.boundary_kind, ctx->g.Re, s);
  return ctx->impl->step(ctx, kVariantProjection, s, 1);
}

int mifgpu_run(mifgpu_ctx *ctx, double t0, int nsteps) {
  if (!ctx || nsteps < 0) return MIFGPU_EINVAL;
  if (nsteps == 0) return MIFGPU_OK;
  if (nsteps > 1 && ctx->prm.boundary_kind == MIFGPU_FIELD_CALLER)
    return fail(ctx, MIFGPU_ENOTSUP,
                "with boundary_kind MIFGPU_FIELD_CALLER the boundary data is set per step: run one step at a time");
  std::vector<double> s((size_t)kSlotSize * nsteps);
  for (int n = 0; n < nsteps; ++n)
    projection_slot(t0 + n * ctx->g.dt, ctx->g.dt, ctx->prm.boundary_kind, ctx->g.Re, s.data() + (size_t)kSlotSize * n);
  return ctx->impl->step(ctx, kVariantProjection, s.data(), nsteps);
}

int mifgpu_timestep_host(mifgpu_ctx *ctx, double t_n, double *u, double *v, double *w, double *p) {
  if (!ctx || !u || !v || !w || !p) return MIFGPU_EINVAL;
  double *h[4] = {u, v, w, p};
  const double *hc[4] = {u, v, w, p};
  const int ids[4] = {0, 1, 2, kP};
  if (int rc = ctx->impl->upload_fields(ctx, ids, hc, 4)) return rc;
  const int rc = mifgpu_timestep(ctx, t_n);
  if (rc != MIFGPU_OK && rc != MIFGPU_ENONFINITE) return rc;
  // a non-finite step still hands its state back, then reports it
  const std::string msg = ctx->err;
  if (int rd = ctx->impl->download_fields(ctx, ids, h, 4)) return rd;
  if (rc != MIFGPU_OK) ctx->err = msg;
  return rc;
}

int mifgpu_timestep_nhn(mifgpu_ctx *ctx, double t_n) {
  if (!ctx) return MIFGPU_EINVAL;
  if (ctx->g.periodic[0] || ctx->g.periodic[1] || ctx->g.periodic[2])
    return fail(ctx, MIFGPU_ENOTSUP, "non-homogeneous Neumann data needs every axis non-periodic");
  double s[kSlotSize];
  projection_slot(t_n, ctx->g.dt, ctx->prm.boundary_kind, ctx->g.Re, s);
  return ctx->impl->step(ctx, kVariantNhn, s, 1);
}

int mifgpu_timestep_velocity(mifgpu_ctx *ctx, double t_n) {
  if (!ctx) return MIFGPU_EINVAL;
  if (ctx->prm.precision == MIFGPU_MIXED_COMPENSATED)
    return fail(ctx, MIFGPU_ENOTSUP, "the velocity-only step runs in MIFGPU_FP64 or MIFGPU_MIXED");
  double s[kSlotSize];
  velocity_slot(t_n, ctx->g.dt, ctx->prm.boundary_kind, ctx->g.Re, s);
  return ctx->impl->step(ctx, kVariantVelocity, s, 1);  // ends with the swap, src/TimestepVelocity.cpp:89
}

int mifgpu_run_velocity(mifgpu_ctx *ctx, double t0, int nsteps) {
  if (!ctx || nsteps < 0) return MIFGPU_EINVAL;
  if (nsteps == 0) return MIFGPU_OK;
  if (ctx->prm.precision == MIFGPU_MIXED_COMPENSATED)
    return fail(ctx, MIFGPU_ENOTSUP, "the velocity-only step runs in MIFGPU_FP64 or MIFGPU_MIXED");
  if (nsteps > 1 && ctx->prm.boundary_kind == MIFGPU_FIELD_CALLER)
    return fail(ctx, MIFGPU_ENOTSUP,
                "with boundary_kind MIFGPU_FIELD_CALLER the boundary data is set per step: run one step at a time");
  std::vector<double> s((size_t)kSlotSize * nsteps);
  for (int n = 0; n < nsteps; ++n)
    velocity_slot(t0 + n * ctx->g.dt, ctx->g.dt, ctx->prm.boundary_kind, ctx->g.Re, s.data() + (size_t)kSlotSize * n);
  return ctx->impl->step(ctx, kVariantVelocity, s.data(), nsteps);
}

int mifgpu_set_boundary_values(mifgpu_ctx *ctx, int slot, const double *u, const double *v, const double *w) {
  if (!ctx || !u || !v || !w || slot < 0 || slot > 3) return MIFGPU_EINVAL;
  const double *vel[3] = {u, v, w};
  return ctx->impl->set_boundary_values(ctx, slot, vel);
}

int mifgpu_set_pressure_gradient_faces(mifgpu_ctx *ctx, int slot, const double *const faces[6]) {
  if (!ctx || !faces || slot < 0 || slot > 3) return MIFGPU_EINVAL;
  for (int f = 0; f < 6; ++f)
    if (!faces[f]) return MIFGPU_EINVAL;
  if (ctx->prm.boundary_kind != MIFGPU_FIELD_CALLER)
    return fail(ctx, MIFGPU_EINVAL, "set_pressure_gradient_faces needs boundary_kind MIFGPU_FIELD_CALLER");
  return ctx->impl->set_gradient_faces(ctx, slot, faces);
}

int mifgpu_solve_pressure_nhn(mifgpu_ctx *ctx, int set, double dt, const double *const faces[6]) {
  if (!ctx || !faces || set < 0 || set > 2 || !(dt != 0)) return MIFGPU_EINVAL;
  for (int f = 0; f < 6; ++f)
    if (!faces[f]) return MIFGPU_EINVAL;
  if (ctx->g.periodic[0] || ctx->g.periodic[1] || ctx->g.periodic[2])
    return fail(ctx, MIFGPU_ENOTSUP, "non-homogeneous Neumann data needs every axis non-periodic");
  if (int rc = ctx->impl->set_gradient_faces(ctx, 0, faces)) return rc;
  return ctx->impl->solve_pressure_nhn(ctx, set, dt);
}

int mifgpu_apply_bc(mifgpu_ctx *ctx, int set, double t) {
  if (!ctx || set < 0 || set > 2) return MIFGPU_EINVAL;
  return ctx->impl->apply_bc(ctx, set, t);
}

int mifgpu_solve_pressure(mifgpu_ctx *ctx, int set, double dt) {
  if (!ctx || set < 0 || set > 2 || !(dt != 0)) return MIFGPU_EINVAL;
  return ctx->impl->solve_pressure(ctx, set, dt, true);
}

int mifgpu_divergence(mifgpu_ctx *ctx, int set, double dt) {
  if (!ctx || set < 0 || set > 2 || !(dt != 0)) return MIFGPU_EINVAL;
  return ctx->impl->solve_pressure(ctx, set, dt, false);
}

int mifgpu_project(mifgpu_ctx *ctx, int set, double dt) {
  if (!ctx || set < 0 || set > 2) return MIFGPU_EINVAL;
  return ctx->impl->project(ctx, set, dt);
}

int mifgpu_adjust_pressure(mifgpu_ctx *ctx, double t) {
  if (!ctx) return MIFGPU_EINVAL;
  if (int rc = needs_family(ctx, "adjust_pressure")) return rc;
  return ctx->impl->adjust_pressure(ctx, t);
}

int mifgpu_error_norms(mifgpu_ctx *ctx, double t, double out[9]) {
  if (!ctx || !out) return MIFGPU_EINVAL;
  if (int rc = needs_family(ctx, "error_norms")) return rc;
  return ctx->impl->error_norms(ctx, t, out);
}

int mifgpu_profile_step(mifgpu_ctx *ctx, double t_n, int reps, double ms_out[MIFGPU_PROF_CLASSES]) {
  if (!ctx || !ms_out || reps < 1) return MIFGPU_EINVAL;
  return ctx->impl->profile_step(ctx, t_n, reps, ms_out);
}

int mifgpu_gradient_ke(mifgpu_ctx *ctx, double t0, int nsteps, int checkpoint_every, const double box[6],
                       double *loss, double *dloss_dalpha, double ms_out[3]) {
  if (!ctx || !box || nsteps < 1 || checkpoint_every < 1) return MIFGPU_EINVAL;
  if (int rc = needs_family(ctx, "the reverse mode")) return rc;
  GradRequest r;
  r.t0 = t0;
  r.nsteps = nsteps;
  r.every = checkpoint_every;
  r.box = box;
  r.loss = loss;
  r.dalpha = dloss_dalpha;
  r.ms = ms_out;
  return ctx->impl->gradient(ctx, r);
}

int mifgpu_backward(mifgpu_ctx *ctx, double t0, int nsteps, int checkpoint_every, const double *seed_u,
                    const double *seed_v, const double *seed_w, const double *seed_p, double *dloss_dalpha,
                    double ms_out[3]) {
  if (!ctx || nsteps < 1 || checkpoint_every < 1) return MIFGPU_EINVAL;
  if (int rc = needs_family(ctx, "the reverse mode")) return rc;
  GradRequest r;
  r.t0 = t0;
  r.nsteps = nsteps;
  r.every = checkpoint_every;
  r.seed[0] = seed_u;
  r.seed[1] = seed_v;
  r.seed[2] = seed_w;
  r.seed[3] = seed_p;
  r.dalpha = dloss_dalpha;
  r.ms = ms_out;
  return ctx->impl->gradient(ctx, r);
}

int mifgpu_download_adjoint(mifgpu_ctx *ctx, int field, double *host) {
  if (!ctx || !host || !(field == 0 || field == 1 || field == 2 || field == kP)) return MIFGPU_EINVAL;
  return ctx->impl->download_adjoint(ctx, field, host);
}

int mifgpu_set_forcing_amplitude(mifgpu_ctx *ctx, double alpha) {
  if (!ctx || !std::isfinite(alpha)) return MIFGPU_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->prm.forcing_amplitude = alpha;
  ctx->impl->drop_graphs();
  return MIFGPU_OK;
}

int mifgpu_velocity_error_norms_noalloc(mifgpu_ctx *ctx, double t, double out[3]) {
  if (!ctx || !out) return MIFGPU_EINVAL;
  if (int rc = needs_family(ctx, "velocity_error_norms_noalloc")) return rc;
  const Geometry &g = ctx->g;
  const int planes = g.E[2] - 2;
  if (planes > kNoAllocMaxPlanes)
    return fail(ctx, MIFGPU_EINVAL,
                "velocity_error_norms_noalloc: " + std::to_string(planes) + " interior z planes exceed the " +
                    std::to_string(kNoAllocMaxPlanes) + " its static scratch holds (n_global[2] at most " +
                    std::to_string(kNoAllocMaxPlanes + 2) + " on a Dirichlet z axis, " +
                    std::to_string(kNoAllocMaxPlanes + 1) + " on a periodic one)");
  int cur = -1;
  CK(cudaGetDevice(&cur));
  if (cur != ctx->device) return fail(ctx, MIFGPU_EINVAL, "velocity_error_norms_noalloc: the context's device is not current");
  double *scratch = nullptr;
  std::string err;
  if (noalloc_scratch(&scratch, err)) return fail(ctx, MIFGPU_ECUDA, err);
  const int kind = ctx->prm.boundary_kind;
  if (ctx->prm.precision == MIFGPU_FP64)
    launch_velocity_errors_noalloc<double>(g, (const double *)ctx->impl->field_ptr(0),
                                           (const double *)ctx->impl->field_ptr(1),
                                           (const double *)ctx->impl->field_ptr(2), kind, t, scratch, ctx->stream,
                                           &ctx->launches, Residual{});
  else
    launch_velocity_errors_noalloc<float>(g, (const float *)ctx->impl->field_ptr(0),
                                          (const float *)ctx->impl->field_ptr(1),
                                          (const float *)ctx->impl->field_ptr(2), kind, t, scratch, ctx->stream,
                                          &ctx->launches, ctx->impl->residual());
  CK(cudaGetLastError());
  double h[3];
  CK(cudaMemcpyAsync(h, scratch + 3 * kNoAllocMaxPlanes, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const double vol = g.h[0] * g.h[1] * g.h[2];
  out[0] = h[0] * vol;
  out[1] = std::sqrt(h[1] * vol);
  out[2] = h[2];
  return MIFGPU_OK;
}

namespace {
ExportSource export_source(mifgpu_ctx *ctx) {
  ExportSource src;
  src.g = ctx->g;
  for (int d = 0; d < 3; ++d) src.size[d] = ctx->prm.size[d];
  src.fp64 = ctx->prm.precision == MIFGPU_FP64;
  src.fetch = [ctx](int id, const int lo[3], const int n[3], double *out) {
    return ctx->impl->fetch_box(ctx, id, lo, n, out);
  };
  return src;
}
int export_result(mifgpu_ctx *ctx, int rc, const std::string &err) {
  if (rc != MIFGPU_OK && !err.empty()) return fail(ctx, rc, err);
  return rc;
}
}  // namespace

int mifgpu_write_vtk(mifgpu_ctx *ctx, const char *filename) {
  if (!ctx || !filename) return MIFGPU_EINVAL;
  std::string err;
  const int rc = export_vtk(export_source(ctx), filename, err);
  return export_result(ctx, rc, err);
}

int mifgpu_write_dat(mifgpu_ctx *ctx, const char *filename, int direction, double x, double y, double z) {
  if (!ctx || !filename) return MIFGPU_EINVAL;
  std::string err;
  const int rc = export_dat(export_source(ctx), filename, direction, x, y, z, err);
  return export_result(ctx, rc, err);
}

int mifgpu_write_vtk_full_mesh(mifgpu_ctx *ctx, const char *filename) {
  if (!ctx || !filename) return MIFGPU_EINVAL;
  std::string err;
  const int rc = export_vtk_full_mesh(export_source(ctx), filename, err);
  return export_result(ctx, rc, err);
}

int mifgpu_launch_count(const mifgpu_ctx *ctx, long long *out) {
  if (!ctx || !out) return MIFGPU_EINVAL;
  *out = ctx->launches;
  return MIFGPU_OK;
}

int mifgpu_device_bytes(const mifgpu_ctx *ctx, size_t *out) {
  if (!ctx || !out) return MIFGPU_EINVAL;
  *out = ctx->impl->bytes();
  return MIFGPU_OK;
}

}  // extern "C"
