// tmap.cuh -- host-side creation of TMA tensor maps (CUtensorMap) through the
// driver entry point, so the library needs no link-time libcuda dependency.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ejoin_internal.cuh"

namespace ejoin {

typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                    const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                    const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                    CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline PFN_encodeTiled get_encode_tiled() {
    static PFN_encodeTiled fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_encodeTiled)p;
        else
            cudaGetLastError();
    }
    return fn;
}

// Row-major [rows][width] matrix of `esize`-byte elements; box of
// box_w elements x box_h rows; the swizzle span equals the box row
// (box_w * esize = 128 or 32 bytes).
inline int make_tmap_2d(CUtensorMap* map, const void* base, CUtensorMapDataType dtype,
                        uint32_t esize, uint64_t width, uint64_t rows, uint32_t box_w,
                        uint32_t box_h) {
    PFN_encodeTiled enc = get_encode_tiled();
    if (!enc) return set_error(EJOIN_ECUDA, "cuTensorMapEncodeTiled entry point unavailable");
    const uint32_t span = box_w * esize;
    if (((uintptr_t)base & 15) || (width * esize) % 16 || (span != 128 && span != 32))
        return set_error(EJOIN_EINTERNAL, "tensor map: misaligned base/stride/box");
    cuuint64_t dims[2] = {width, rows};
    cuuint64_t strides[1] = {width * esize};
    cuuint32_t box[2] = {box_w, box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, dtype, 2, const_cast<void*>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE,
                     span == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_32B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(EJOIN_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return EJOIN_OK;
}

}  // namespace ejoin
