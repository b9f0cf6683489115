// hyc_tmap.cpp -- host-side TMA descriptors, see hyc_tmap.h.
#include "hyc_tmap.h"

#include <cuda_runtime.h>

namespace hyc {

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

}  // namespace

bool tmap_available() { return encode_fn() != nullptr; }

bool tmap_encode3(CUtensorMap *m, const void *base, int es, long long w, long long h, long long ld1, long long sl,
                  long long nz, int bx, int by) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || !base || (es != 4 && es != 8) || w < 1 || h < 1 || nz < 1 || ld1 < w) return false;
  if (((uintptr_t)base & 15) != 0 || (ld1 * es) % 16 != 0 || (sl * es) % 16 != 0 || ((long long)bx * es) % 16 != 0)
    return false;
  cuuint64_t dims[3] = {(cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)nz};
  cuuint64_t strides[2] = {(cuuint64_t)(ld1 * es), (cuuint64_t)(sl * es)};
  cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt = es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  return fn(m, dt, 3, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace hyc
