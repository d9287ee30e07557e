// Velocity error norms without any allocation (sm_103a): a deterministic
// two-pass reduction whose partial sums live in one file-scope device array
// instead of memory the context allocates. The per-point arithmetic is that
// of velocity_error_kernel (src/Norms.cpp:11-47): velocity averaged to the
// interior nodes, compared with the analytic family in double.
#include <algorithm>
#include <mutex>

#include "analytic.cuh"
#include "noalloc.cuh"

namespace mifgpu {

namespace {

constexpr int kNT = 256;
constexpr int kMaxDevices = 64;

// [3 * k .. 3 * k + 2]: slot k's (sum |e|, sum e^2, max |e|), one slot per
// (interior plane, chunk);
// [3 * kNoAllocMaxPlanes .. + 2]: the totals.
static __device__ __align__(256) double g_norm_scratch[3 * (kNoAllocMaxPlanes + 1)];

// Block-wide (sum, sum, max) in a fixed order; the result is valid in thread 0.
__device__ void block_sum2_max(double &a, double &b, double &m) {
  __shared__ double sa[kNT / 32], sb[kNT / 32], sm[kNT / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sa[wid] = a, sb[wid] = b, sm[wid] = m;
  __syncthreads();
  if (wid == 0) {
    a = lane < kNT / 32 ? sa[lane] : 0.0;
    b = lane < kNT / 32 ? sb[lane] : 0.0;
    m = lane < kNT / 32 ? sm[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    }
  }
}

// Block b takes chunk b % chunks of interior plane 1 + b / chunks: the
// points [c len, (c + 1) len) of the plane's ni x nj interior, x fastest.
// I: the index type of a plane's points (32-bit where the plane fits).
template <typename T, typename I>
__global__ void __launch_bounds__(kNT) velocity_error_plane_kernel(Geometry g, const T *u, const T *v, const T *w,
                                                                   int kind, double t, int chunks, I len,
                                                                   double *part, Residual res) {
  const I ni = (I)(g.E[0] - 2), n = ni * (I)(g.E[1] - 2);
  const long k = 1 + blockIdx.x / chunks;
  const I c = (I)(blockIdx.x % chunks), end = n < (c + 1) * len ? n : (c + 1) * len;
  double a = 0, b = 0, m = 0;
  for (I id = c * len + threadIdx.x; id < end; id += kNT) {
    const long i = 1 + (long)(id % ni), j = 1 + (long)(id / ni);
    const long q = g.idx(i, j, k);
    const double x = g.origin[0] + (double)(g.base[0] + i) * g.h[0];
    const double y = g.origin[1] + (double)(g.base[1] + j) * g.h[1];
    const double z = g.origin[2] + (double)(g.base[2] + k) * g.h[2];
    // the compensated state's value is hi + residual
    auto val = [&](const T *f, int c, long qq) {
      return res.on() ? (double)f[qq] + (double)__bfloat162float(res.c[c][qq]) : (double)f[qq];
    };
    const double iu = (val(u, 0, q) + val(u, 0, q + 1)) / 2.0;
    const double iv = (val(v, 1, q) + val(v, 1, q + g.sy())) / 2.0;
    const double iw = (val(w, 2, q) + val(w, 2, q + g.sz())) / 2.0;
    const double eu = analytic_value<double>(kind, 0, t, x, y, z, g.Re) - iu;
    const double ev = analytic_value<double>(kind, 1, t, x, y, z, g.Re) - iv;
    const double ew = analytic_value<double>(kind, 2, t, x, y, z, g.Re) - iw;
    a += sqrt(eu * eu + ev * ev + ew * ew);
    b += eu * eu + ev * ev + ew * ew;
    m = fmax(m, fmax(fmax(fabs(eu), fabs(ev)), fabs(ew)));
  }
  block_sum2_max(a, b, m);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x + 0] = a;
    part[3 * blockIdx.x + 1] = b;
    part[3 * blockIdx.x + 2] = m;
  }
}

__global__ void __launch_bounds__(kNT) plane_totals_kernel(const double *part, int slots, double *out) {
  double a = 0, b = 0, m = 0;
  for (int k = threadIdx.x; k < slots; k += kNT) {
    a += part[3 * k + 0];
    b += part[3 * k + 1];
    m = fmax(m, part[3 * k + 2]);
  }
  block_sum2_max(a, b, m);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
    out[2] = m;
  }
}

}  // namespace

// The unique id of the current context (cuCtxGetId, reached through the
// runtime's driver entry point so the library needs no libcuda link), or 0
// if the driver cannot tell.
unsigned long long current_context_id() {
  using GetId = int (*)(void *, unsigned long long *);  // CUresult cuCtxGetId(CUcontext, unsigned long long *)
  static GetId fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (GetId) nullptr;
    return reinterpret_cast<GetId>(p);
  }();
  unsigned long long id = 0;
  if (!fn || fn(nullptr, &id) != 0) return 0;
  return id;
}

int noalloc_scratch(double **out, std::string &err) {
  // Per device: the context the address was looked up in and the address. A
  // new context on the device (after cudaDeviceReset, say) reloads the
  // module and may move the array, so the lookup is repeated for it.
  struct Entry {
    unsigned long long ctx;
    void *addr;
  };
  static std::mutex mu;
  static Entry cache[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return -2;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    err = "device index beyond the scratch address cache";
    return -2;
  }
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(mu);
  if (!cache[dev].addr || cache[dev].ctx != ctx) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_norm_scratch);
    if (e != cudaSuccess) {
      err = std::string("cudaGetSymbolAddress of the norm scratch: ") + cudaGetErrorString(e);
      return -2;
    }
    cache[dev] = Entry{ctx, p};
  }
  *out = static_cast<double *>(cache[dev].addr);
  return 0;
}

template <typename T>
void launch_velocity_errors_noalloc(const Geometry &g, const T *u, const T *v, const T *w, int field_kind, double t,
                                    double *scratch, cudaStream_t s, long long *launches, const Residual &res) {
  const int planes = g.E[2] - 2;
  const long n = (long)(g.E[0] - 2) * (g.E[1] - 2);
  const long by_points = std::max(1L, n / 1024);
  const int chunks = (int)std::max(1L, std::min((long)(kNoAllocMaxPlanes / std::max(planes, 1)), by_points));
  const long len = (n + chunks - 1) / chunks;
  const unsigned blocks = (unsigned)(planes * chunks);
  if (n + len + kNT < (1L << 31))  // every index the chunk loop forms fits an int
    velocity_error_plane_kernel<T, int>
        <<<blocks, kNT, 0, s>>>(g, u, v, w, field_kind, t, chunks, (int)len, scratch, res);
  else
    velocity_error_plane_kernel<T, long><<<blocks, kNT, 0, s>>>(g, u, v, w, field_kind, t, chunks, len, scratch, res);
  plane_totals_kernel<<<1, kNT, 0, s>>>(scratch, planes * chunks, scratch + 3 * kNoAllocMaxPlanes);
  if (launches) *launches += 2;
}

template void launch_velocity_errors_noalloc<float>(const Geometry &, const float *, const float *, const float *,
                                                    int, double, double *, cudaStream_t, long long *,
                                                    const Residual &);
template void launch_velocity_errors_noalloc<double>(const Geometry &, const double *, const double *,
                                                     const double *, int, double, double *, cudaStream_t,
                                                     long long *, const Residual &);

}  // namespace mifgpu
