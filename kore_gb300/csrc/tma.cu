// Host-side encoding of the tensor maps that the TMA copies of the sweep and of the
// tensor-core GEMMs read.  The encoder is the driver's cuTensorMapEncodeTiled, fetched
// at run time through the runtime API (no link against libcuda).
#include "kore_tma.cuh"
#include <cstdio>
namespace {
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled_fn() {
    static EncodeTiledFn fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<EncodeTiledFn>(f);
    }();
    return fn;
}
}  // namespace

int kore_encode_block_map(CUtensorMap *map, const void *base, int real_bytes, int S, int64_t nblk, int nshift,
                          int64_t shift_stride, int box_rows, int box_cols) {
    EncodeTiledFn fn = encode_tiled_fn();
    if (!fn) {
        std::fprintf(stderr, "kore: cuTensorMapEncodeTiled is not available from the driver\n");
        return KORE_ECUDA;
    }
    const cuuint64_t cb = 2 * (cuuint64_t)real_bytes;   // bytes of one complex entry
    const cuuint64_t dims[4] = {2 * (cuuint64_t)S, (cuuint64_t)S, (cuuint64_t)nblk, (cuuint64_t)nshift};
    const cuuint64_t strides[3] = {cb * S, cb * S * S, cb * (cuuint64_t)shift_stride};
    const cuuint32_t box[4] = {2 * (cuuint32_t)box_rows, (cuuint32_t)box_cols, 1, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = fn(map, real_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4,
                          const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        std::fprintf(stderr, "kore: cuTensorMapEncodeTiled failed (%d): S=%d blocks=%lld shifts=%d\n", (int)r, S,
                     (long long)nblk, nshift);
        return KORE_ECUDA;
    }
    return KORE_OK;
}

int kore_encode_f32_3d(CUtensorMap *map, const void *base, const uint64_t dims[3], const uint64_t strides[2],
                       const uint32_t box[3], int swizzle128) {
    EncodeTiledFn fn = encode_tiled_fn();
    if (!fn) {
        std::fprintf(stderr, "kore: cuTensorMapEncodeTiled is not available from the driver\n");
        return KORE_ECUDA;
    }
    const cuuint64_t d[3] = {dims[0], dims[1], dims[2]};
    const cuuint64_t st[2] = {strides[0], strides[1]};
    const cuuint32_t b[3] = {box[0], box[1], box[2]};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(base), d, st, b, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE,
                          swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        std::fprintf(stderr, "kore: cuTensorMapEncodeTiled (3-D float) failed (%d)\n", (int)r);
        return KORE_ECUDA;
    }
    return KORE_OK;
}
