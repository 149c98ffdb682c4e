// k_misc.cu -- tile-pair work lists, totals and count scatter.
//
// Work list: the upper-triangle 128x128 tile pairs (I <= J) in a blocked
// order -- super-blocks of SB x SB tile pairs, super-blocks in row-major
// triangular order -- so that the CTAs running concurrently touch a few MB of
// operand rows that stay resident in L2.  The list is built by ordered
// stream compaction over the candidate index space; the same pass drops tile
// pairs the learned projection proves empty (see k_learn.cu for the bound).
#include "ejoin_internal.cuh"

namespace ejoin {
namespace {

constexpr uint32_t SB = 16;           // super-block edge (tiles)
constexpr int CAND_PER_THREAD = 16;
constexpr int CAND_THREADS = 256;
constexpr uint64_t CAND_PER_BLOCK = (uint64_t)CAND_PER_THREAD * CAND_THREADS;

struct PruneArgs {
    const double* lo;    // [ntiles][k] lower corners of the projected boxes (may be null)
    const double* hi;    // [ntiles][k]
    uint32_t k;
    double thr;          // skip the pair when the squared box gap exceeds thr
};

__device__ __forceinline__ bool candidate(uint64_t c, uint64_t nT, uint64_t nS, const PruneArgs& p,
                                          uint2& out) {
    const uint64_t sp = c / (SB * SB);
    const uint32_t r = (uint32_t)(c % (SB * SB));
    uint64_t SI, SJ;
    tri_decode(sp, nS, SI, SJ);
    const uint64_t I = SI * SB + r / SB, J = SJ * SB + r % SB;
    if (I >= nT || J >= nT || I > J) return false;
    if (p.lo) {
        // squared gap between the projected boxes, rounded down (see k_learn.cu)
        double g2 = 0.0;
        for (uint32_t a = 0; a < p.k; ++a) {
            const double l1 = p.lo[I * p.k + a], h1 = p.hi[I * p.k + a];
            const double l2 = p.lo[J * p.k + a], h2 = p.hi[J * p.k + a];
            const double gap = fmax(0.0, fmax(__dsub_rd(l2, h1), __dsub_rd(l1, h2)));
            g2 = __fma_rd(gap, gap, g2);
        }
        if (g2 > p.thr) return false;
    }
    out = make_uint2((uint32_t)I, (uint32_t)J);
    return true;
}

__global__ void __launch_bounds__(CAND_THREADS) count_kernel(uint64_t ncand, uint64_t nT,
                                                             uint64_t nS, PruneArgs p,
                                                             uint32_t* block_counts) {
    uint32_t cnt = 0;
    const uint64_t base = blockIdx.x * CAND_PER_BLOCK + (uint64_t)threadIdx.x * CAND_PER_THREAD;
    for (int e = 0; e < CAND_PER_THREAD; ++e) {
        const uint64_t c = base + e;
        uint2 w;
        if (c < ncand && candidate(c, nT, nS, p, w)) ++cnt;
    }
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    __shared__ uint32_t ws[CAND_THREADS / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x / 32] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int i = 0; i < CAND_THREADS / 32; ++i) s += ws[i];
        block_counts[blockIdx.x] = s;
    }
}

// exclusive scan of block counts (single block, sequential chunks)
__global__ void scan_kernel(const uint32_t* in, uint64_t n, uint64_t* out, uint64_t* total) {
    __shared__ uint64_t carry;
    __shared__ uint64_t buf[1024];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint64_t base = 0; base < n; base += 1024) {
        const uint64_t i = base + threadIdx.x;
        buf[threadIdx.x] = i < n ? in[i] : 0;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            uint64_t v = threadIdx.x >= (unsigned)o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += v;
            __syncthreads();
        }
        const uint64_t incl = buf[threadIdx.x];
        const uint64_t own = i < n ? in[i] : 0;
        if (i < n) out[i] = carry + incl - own;
        __syncthreads();
        if (threadIdx.x == 1023) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(CAND_THREADS) write_kernel(uint64_t ncand, uint64_t nT,
                                                             uint64_t nS, PruneArgs p,
                                                             const uint64_t* offsets, uint2* out) {
    const uint64_t base = blockIdx.x * CAND_PER_BLOCK + (uint64_t)threadIdx.x * CAND_PER_THREAD;
    uint32_t cnt = 0;
    for (int e = 0; e < CAND_PER_THREAD; ++e) {
        const uint64_t c = base + e;
        uint2 w;
        if (c < ncand && candidate(c, nT, nS, p, w)) ++cnt;
    }
    // block exclusive scan of cnt (thread order == candidate order)
    __shared__ uint32_t ws[CAND_THREADS / 32];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x / 32;
    uint32_t incl = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += v;
    }
    if (lane == 31) ws[wid] = incl;
    __syncthreads();
    uint32_t wbase = 0;
    for (uint32_t i = 0; i < wid; ++i) wbase += ws[i];
    uint64_t pos = offsets[blockIdx.x] + wbase + incl - cnt;
    for (int e = 0; e < CAND_PER_THREAD; ++e) {
        const uint64_t c = base + e;
        uint2 w;
        if (c < ncand && candidate(c, nT, nS, p, w)) out[pos++] = w;
    }
}

__global__ void sum_counts_kernel(const int32_t* counts, uint64_t n, unsigned long long* total) {
    unsigned long long s = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        s += (unsigned long long)(uint32_t)counts[i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(total, s);
}

__global__ void scatter_counts_kernel(const int32_t* src, const uint32_t* perm, uint64_t n,
                                      int32_t* dst) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) dst[perm[i]] = src[i];
}

}  // namespace

// Builds the ordered list of surviving tile pairs.  lo/hi may be null (plain
// join).  *nwork_out receives the count; `work` is allocated here.
int build_worklist(uint64_t nT, const double* lo, const double* hi, uint32_t k, double thr,
                   DBuf<uint2>& work, uint64_t* nwork_out, uint64_t* ncand_out, cudaStream_t s) {
    *nwork_out = 0;
    if (nT == 0) return EJOIN_OK;
    const uint64_t nS = (nT + SB - 1) / SB;
    const uint64_t ncand = nS * (nS + 1) / 2 * SB * SB;
    if (ncand_out) *ncand_out = ncand;
    const uint64_t nblocks = (ncand + CAND_PER_BLOCK - 1) / CAND_PER_BLOCK;
    if (nblocks > 0x7fffffffull) return set_error(EJOIN_EUNSUPPORTED, "work list too large");
    PruneArgs p{lo, hi, k, thr};
    DBuf<uint32_t> bc;
    DBuf<uint64_t> off;
    EJ_TRY(bc.alloc(nblocks, s, "work-list block counts"));
    EJ_TRY(off.alloc(nblocks + 1, s, "work-list offsets"));
    count_kernel<<<(unsigned)nblocks, CAND_THREADS, 0, s>>>(ncand, nT, nS, p, bc.p);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    scan_kernel<<<1, 1024, 0, s>>>(bc.p, nblocks, off.p, off.p + nblocks);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    uint64_t total = 0;
    EJ_CUDA(cudaMemcpyAsync(&total, off.p + nblocks, sizeof total, cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    EJ_TRY(work.alloc(total ? total : 1, s, "work list"));
    if (total) {
        write_kernel<<<(unsigned)nblocks, CAND_THREADS, 0, s>>>(ncand, nT, nS, p, off.p, work.p);
        EJ_CUDA(cudaGetLastError());
        note_launch();
    }
    *nwork_out = total;
    return EJOIN_OK;
}

int sum_counts(const int32_t* counts, uint64_t n, unsigned long long* dev_total, cudaStream_t s) {
    if (n == 0) return EJOIN_OK;
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    sum_counts_kernel<<<(unsigned)blocks, 256, 0, s>>>(counts, n, dev_total);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

int scatter_counts(const int32_t* src, const uint32_t* perm, uint64_t n, int32_t* dst,
                   cudaStream_t s) {
    if (n == 0) return EJOIN_OK;
    scatter_counts_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, perm, n, dst);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

}  // namespace ejoin
