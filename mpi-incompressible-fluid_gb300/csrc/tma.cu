// Host side of the TMA tile loads (tma.cuh): tensor maps of padded fields.
#include <cudaTypedefs.h>

#include <mutex>

#include "tma.cuh"

namespace mifgpu {

namespace {

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library links the runtime only).
PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

}  // namespace

bool make_field_map(CUtensorMap *map, const void *base, int elem, long PX, long PY, long PZ, int bx, int by) {
  const long dims[3] = {PX, PY, PZ}, strides[2] = {PX * elem, PX * PY * elem};
  return make_map_3d(map, base, elem, dims, strides, bx, by);
}

bool make_map_3d(CUtensorMap *map, const void *base, int elem, const long dims_[3], const long strides_[2], int bx,
                 int by) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
  if (!enc || (elem != 4 && elem != 8)) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)dims_[0], (cuuint64_t)dims_[1], (cuuint64_t)dims_[2]};
  const cuuint64_t strides[2] = {(cuuint64_t)strides_[0], (cuuint64_t)strides_[1]};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1u};
  const cuuint32_t step[3] = {1u, 1u, 1u};
  return enc(map, elem == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
             const_cast<void *>(base), dims, strides, box, step, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace mifgpu
