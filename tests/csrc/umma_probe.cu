// umma_probe.cu -- GPU self-test of the tcgen05 building blocks (test only).
//
// One CTA computes one 128 x 128 FP32 tile D = A * B^T from K-major operand
// tiles loaded by TMA with the 128-byte swizzle, exactly as the join's Gram
// kernel does, and writes D to global memory so the test can compare it with
// a host product.  It pins the instruction / shared-memory descriptor
// encodings, the swizzled k-advance, the tensor-memory lane/column layout of
// the 32x32b loads and the FP32 accumulation behaviour the screen's error
// bound relies on.  All waits are bounded (umma_ptx.cuh).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "tmap.cuh"
#include "umma_ptx.cuh"

using namespace ejoin;

namespace {

constexpr int kSlabBytes = 128 * 128;  // 128 rows x 128 bytes

__global__ void __launch_bounds__(128, 1) probe_kernel(const __grid_constant__ CUtensorMap ta,
                                                       const __grid_constant__ CUtensorMap tb,
                                                       int nslab, int fmt, int mode, float* D,
                                                       DevStatus* st) {
    extern __shared__ uint8_t smraw[];
    uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = sm;
    uint8_t* sB = sm + nslab * kSlabBytes;
    __shared__ uint64_t bar_full, bar_mma;
    __shared__ uint32_t tmem_base;
    const int warp = threadIdx.x / 32, lane = threadIdx.x & 31;
    if (warp == 0) {
        ptx::tmem_alloc(&tmem_base, 128);
        ptx::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        ptx::mbar_init(&bar_full, 1);
        ptx::mbar_init(&bar_mma, 1);
        ptx::fence_barrier_init();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = tmem_base;
    bool ok = true;
    if (threadIdx.x == 0) {
        if (mode == 2) {
            ptx::mbar_arrive_expect_tx(&bar_full, 2u * 128 * 32);
            ptx::tma_load_2d(sA, &ta, 0, 0, &bar_full);
            ptx::tma_load_2d(sB, &tb, 16, 0, &bar_full);
        } else {
            ptx::mbar_arrive_expect_tx(&bar_full, 2u * nslab * kSlabBytes);
            const int ew = (fmt == 2) ? 128 : 64;  // elements per 128-byte row
            for (int s = 0; s < nslab; ++s) {
                ptx::tma_load_2d(sA + s * kSlabBytes, &ta, s * ew, 0, &bar_full);
                ptx::tma_load_2d(sB + s * kSlabBytes, &tb, s * ew, 0, &bar_full);
            }
        }
        ok = ptx::mbar_wait(&bar_full, 0, st, 1);
        if (ok) {
            ptx::tc_fence_after();
            const uint32_t idesc = (fmt == 2) ? ptx::idesc_f32acc(0, 0, 128, 128)
                                              : ptx::idesc_f32acc(fmt == 1 ? 1 : 0, fmt == 1 ? 1 : 0, 128, 128);
            if (mode == 2) {
                // 32-byte swizzled [128][16] tiles: A from box x=0 of ta, B from box x=16 of tb
                uint64_t ad = ptx::sdesc_sw32(ptx::smem_u32(sA));
                uint64_t bd = ptx::sdesc_sw32(ptx::smem_u32(sB));
                ptx::mma_f16(tmem, ad, bd, idesc, 0);
            } else if (mode == 0) {
                for (int s = 0; s < nslab; ++s)
                    for (int kk = 0; kk < 4; ++kk) {
                        uint64_t ad = ptx::sdesc_sw128(ptx::smem_u32(sA + s * kSlabBytes)) + 2 * kk;
                        uint64_t bd = ptx::sdesc_sw128(ptx::smem_u32(sB + s * kSlabBytes)) + 2 * kk;
                        if (fmt == 2) ptx::mma_f8(tmem, ad, bd, idesc, (s | kk) != 0);
                        else ptx::mma_f16(tmem, ad, bd, idesc, (s | kk) != 0);
                    }
            } else {
                // one K step: A at byte 0 of slab 0, B at byte 32 of slab 0
                uint64_t ad = ptx::sdesc_sw128(ptx::smem_u32(sA));
                uint64_t bd = ptx::sdesc_sw128(ptx::smem_u32(sB)) + 2;
                if (fmt == 2) ptx::mma_f8(tmem, ad, bd, idesc, 0);
                else ptx::mma_f16(tmem, ad, bd, idesc, 0);
            }
            ptx::mma_commit(&bar_mma);
        }
    }
    __syncthreads();
    ok = ptx::mbar_wait(&bar_mma, 0, st, 2);
    if (ok) {
        ptx::tc_fence_after();
        for (int c = 0; c < 4; ++c) {
            uint32_t r[32];
            ptx::tmem_ld_32x32b_x32(tmem + ((uint32_t)(warp * 32) << 16) + 32 * c, r);
            ptx::tmem_ld_wait();
            const int row = warp * 32 + lane;
            for (int j = 0; j < 32; ++j) D[row * 128 + 32 * c + j] = __uint_as_float(r[j]);
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 0) ptx::tmem_dealloc(tmem, 128);
}

}  // namespace

extern "C" int umma_probe_gram(const void* A, const void* B, int nslab, int fmt, int mode,
                               float* D_host, unsigned* timeout_out) {
    if (nslab < 1 || nslab > 4) return -1;
    const size_t bytes = (size_t)128 * 128 * nslab;
    void *dA = nullptr, *dB = nullptr;
    float* dD = nullptr;
    DevStatus* dst = nullptr;
    int rc = 0;
    CUtensorMap ma, mb;
    const CUtensorMapDataType dt = fmt == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                   : fmt == 1 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                              : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    const uint32_t es = fmt == 2 ? 1 : 2;
    const uint64_t width = bytes / 128 / es;
    const size_t smem = 2 * bytes + 1024;
    DevStatus hst = {};
    if (cudaMalloc(&dA, bytes) || cudaMalloc(&dB, bytes) || cudaMalloc(&dD, 128 * 128 * 4) ||
        cudaMalloc(&dst, sizeof(DevStatus))) { rc = -2; goto done; }
    cudaMemcpy(dA, A, bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, bytes, cudaMemcpyHostToDevice);
    cudaMemset(dD, 0, 128 * 128 * 4);
    cudaMemset(dst, 0, sizeof(DevStatus));
    if (mode == 2) {
        // [128][32] 16-bit matrices, boxes of 16 elements (32 bytes)
        if (make_tmap_2d(&ma, dA, dt, es, 32, 128, 16, 128) ||
            make_tmap_2d(&mb, dB, dt, es, 32, 128, 16, 128)) { rc = -3; goto done; }
    } else if (make_tmap_2d(&ma, dA, dt, es, width, 128, 128 / es, 128) ||
               make_tmap_2d(&mb, dB, dt, es, width, 128, 128 / es, 128)) { rc = -3; goto done; }
    if (cudaFuncSetAttribute(probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) { rc = -4; goto done; }
    probe_kernel<<<1, 128, smem>>>(ma, mb, nslab, fmt, mode, dD, dst);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) { rc = -5; goto done; }
    cudaMemcpy(D_host, dD, 128 * 128 * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&hst, dst, sizeof hst, cudaMemcpyDeviceToHost);
    if (timeout_out) *timeout_out = hst.timeout;
    if (hst.timeout) rc = -6;
done:
    cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(dst);
    return rc;
}
