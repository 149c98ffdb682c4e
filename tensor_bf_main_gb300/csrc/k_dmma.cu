// k_dmma.cu -- plain FP64 tensor-core join: DMMA Gram tiles with a fused
// screen epilogue (EJOIN_FP64_DMMA).
//
// Re-designs the reference's distanceCalculationBruteForceTensorDouble
// (kernel_join.cu:530-677).  The reference gives each warp 8 queries x 8
// candidates, loads the candidate fragment straight from global memory,
// stores every 8x8x4 partial product to shared memory and re-accumulates it
// in scalar code, then takes sqrt(|d2|) <= eps and bumps one global counter
// per hit.  Here a CTA owns one 64x64 tile pair (I <= J) of the upper
// triangle, both row blocks are staged in shared memory with cp.async (two
// stages), every warp keeps a 32x32 accumulator block in registers across
// the whole k loop (mma.sync m8n8k4 f64), and the epilogue classifies each
// Gram entry G against per-row thresholds:
//     in   : G >= h_i + h_j      (certainly d2 <= T)
//     out  : G <  g_i + g_j      (certainly d2 >  T)
//     band : otherwise           -> FP64 recheck with the reference arithmetic
// so the counts are exact.  h and g come from k_prep.cu.
#include "ejoin_internal.cuh"

namespace ejoin {
namespace {

constexpr int TB = 64;
constexpr int KC = 32;
constexpr int PITCH = KC + 4;  // doubles; 288 B rows keep cp.async 16-B aligned
constexpr int STAGE_DOUBLES = 2 * TB * PITCH;
constexpr int SMEM_BYTES = 2 * STAGE_DOUBLES * 8;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ void load_stage(double* sm, const double* __restrict__ Y, uint32_t dp,
                                           uint64_t I, uint64_t J, uint32_t k0) {
    // A rows then B rows; 64 rows x 32 doubles each = 1024 16-B chunks per side
    for (int c = threadIdx.x; c < 2 * TB * (KC / 2); c += blockDim.x) {
        int side = c / (TB * (KC / 2));
        int rem = c % (TB * (KC / 2));
        int r = rem / (KC / 2), q = rem % (KC / 2);
        uint64_t row = (side ? J : I) * TB + r;
        cp_async16(sm + side * TB * PITCH + r * PITCH + 2 * q, Y + row * dp + k0 + 2 * q);
    }
}

__device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(128) dmma_join_kernel(const double* __restrict__ Y, uint32_t dp,
                                                        uint64_t nT, uint64_t tiles,
                                                        const double* __restrict__ h,
                                                        const double* __restrict__ g,
                                                        int32_t* counts, BandPair* band,
                                                        uint64_t band_cap, DevStatus* st) {
    extern __shared__ __align__(16) double smem[];
    __shared__ int rowc[TB], colc[TB];
    const uint64_t t = blockIdx.x + (uint64_t)blockIdx.y * gridDim.x;
    if (t >= tiles) return;
    uint64_t I, J;
    tri_decode(t, nT, I, J);
    const int warp = threadIdx.x / 32, lane = threadIdx.x & 31;
    const int wr = warp / 2, wc = warp % 2;
    const int gq = lane >> 2, t4 = lane & 3;
    if (threadIdx.x < TB) {
        rowc[threadIdx.x] = 0;
        colc[threadIdx.x] = 0;
    }
    double acc[4][4][2];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int nn = 0; nn < 4; ++nn) acc[m][nn][0] = acc[m][nn][1] = 0.0;

    const uint32_t nk = dp / KC;
    load_stage(smem, Y, dp, I, J, 0);
    cp_async_commit();
    for (uint32_t kc = 0; kc < nk; ++kc) {
        if (kc + 1 < nk) {
            load_stage(smem + ((kc + 1) & 1) * STAGE_DOUBLES, Y, dp, I, J, (kc + 1) * KC);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const double* SA = smem + (kc & 1) * STAGE_DOUBLES;
        const double* SB = SA + TB * PITCH;
#pragma unroll
        for (int ks = 0; ks < KC / 4; ++ks) {
            double a[4], b[4];
#pragma unroll
            for (int m = 0; m < 4; ++m) a[m] = SA[(wr * 32 + 8 * m + gq) * PITCH + ks * 4 + t4];
#pragma unroll
            for (int nn = 0; nn < 4; ++nn) b[nn] = SB[(wc * 32 + 8 * nn + gq) * PITCH + ks * 4 + t4];
#pragma unroll
            for (int m = 0; m < 4; ++m)
#pragma unroll
                for (int nn = 0; nn < 4; ++nn) dmma(acc[m][nn][0], acc[m][nn][1], a[m], b[nn]);
        }
        __syncthreads();
    }

    // ---- epilogue: classify, count, queue the band
    const bool diag = (I == J);
    double hr[4], gr[4], hc[8], gc[8];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        uint64_t i = I * TB + wr * 32 + 8 * m + gq;
        hr[m] = h[i];
        gr[m] = g[i];
    }
#pragma unroll
    for (int nn = 0; nn < 4; ++nn)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            uint64_t j = J * TB + wc * 32 + 8 * nn + 2 * t4 + e;
            hc[2 * nn + e] = h[j];
            gc[2 * nn + e] = g[j];
        }
    unsigned nband = 0;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int nn = 0; nn < 4; ++nn)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                double G = acc[m][nn][e];
                bool in = __dsub_rn(G, hc[2 * nn + e]) >= hr[m];
                bool out = __dsub_rn(G, gc[2 * nn + e]) < gr[m];
                if (in) {
                    atomicAdd(&rowc[wr * 32 + 8 * m + gq], 1);
                    if (!diag) atomicAdd(&colc[wc * 32 + 8 * nn + 2 * t4 + e], 1);
                }
                nband += (!in && !out);
            }
    if (__any_sync(0xffffffffu, nband != 0)) {
        unsigned long long slot = band_reserve(st, nband);
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int nn = 0; nn < 4; ++nn)
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    double G = acc[m][nn][e];
                    bool in = __dsub_rn(G, hc[2 * nn + e]) >= hr[m];
                    bool out = __dsub_rn(G, gc[2 * nn + e]) < gr[m];
                    if (!in && !out) {
                        if (slot < band_cap) {
                            BandPair bp;
                            bp.i = (uint32_t)(I * TB + wr * 32 + 8 * m + gq);
                            bp.j = (uint32_t)(J * TB + wc * 32 + 8 * nn + 2 * t4 + e) |
                                   (diag ? 0u : kBandBoth);
                            band[slot] = bp;
                        }
                        ++slot;
                    }
                }
    }
    __syncthreads();
    if (threadIdx.x < TB) {
        if (rowc[threadIdx.x]) atomicAdd(&counts[I * TB + threadIdx.x], rowc[threadIdx.x]);
        if (colc[threadIdx.x]) atomicAdd(&counts[J * TB + threadIdx.x], colc[threadIdx.x]);
    }
}

}  // namespace

int launch_dmma_join(const double* Y, uint64_t n_pad, uint32_t dp, const double* h,
                     const double* g, int32_t* counts, BandPair* band, uint64_t band_cap,
                     DevStatus* st, cudaStream_t s) {
    if (n_pad == 0) return EJOIN_OK;
    if (n_pad % TB || dp % KC) return set_error(EJOIN_EINTERNAL, "dmma: bad padding");
    EJ_CUDA(cudaFuncSetAttribute(dmma_join_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 SMEM_BYTES));
    const uint64_t nT = n_pad / TB;
    const uint64_t tiles = nT * (nT + 1) / 2;
    const uint64_t gx = tiles < 1048576ull ? tiles : 1048576ull;
    const uint64_t gy = (tiles + gx - 1) / gx;
    if (gy > 65535) return set_error(EJOIN_EUNSUPPORTED, "dmma: too many tile pairs");
    dmma_join_kernel<<<dim3((unsigned)gx, (unsigned)gy), 128, SMEM_BYTES, s>>>(
        Y, dp, nT, tiles, h, g, counts, band, band_cap, st);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

}  // namespace ejoin
