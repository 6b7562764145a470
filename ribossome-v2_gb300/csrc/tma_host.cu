// Host side of the TMA tile loads: tensor-map encoding through the driver
// entry point (the library does not link libcuda directly).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <string.h>

#include <mutex>

#include "ribo_tma.cuh"

namespace ribo {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

bool make_tensor_map_2d(CUtensorMap* out, void* base, CUtensorMapDataType type, int elem_bytes, uint64_t w, uint64_t h,
                        uint64_t pitch_elems, uint32_t box_w, uint32_t box_h) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0) return false;
  if ((pitch_elems * elem_bytes) % 16 != 0) return false;
  if ((box_w * (uint32_t)elem_bytes) % 16 != 0 || box_w > 256 || box_h > 256) return false;
  cuuint64_t dims[2] = {w, h};
  cuuint64_t strides[1] = {pitch_elems * (cuuint64_t)elem_bytes};
  cuuint32_t box[2] = {box_w, box_h};
  cuuint32_t estr[2] = {1, 1};
  memset(out, 0, sizeof *out);
  CUresult r = fn(out, type, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace ribo
