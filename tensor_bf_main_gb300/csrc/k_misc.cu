// k_misc.cu -- tile-pair work lists, totals and count scatter.
//
// Work list: blocks of one 128-row tile I x two 128-column tiles (Ja, Jb)
// covering the upper-triangle tile pairs (I <= J), in a blocked order --
// super-blocks of SB x SB tiles, super-blocks in row-major triangular order
// -- so that the CTAs running concurrently touch a few MB of operand rows
// that stay resident in L2.  Each entry carries a 2-bit mask of its active
// halves (tile pairs in the upper triangle, below the last data tile, and not
// proven empty by the learned projection; see k_learn.cu for the bound).
// The two column tiles of a block need not be adjacent: a row's active tiles
// within a super-block are paired, so that a block's second half is inactive
// only for the row's last, odd tile (a 128 x 128 MMA costs as much as a
// 128 x 256 one, so two lone tiles in one block halve their cost).
#include <cub/cub.cuh>

#include "ejoin_internal.cuh"

namespace ejoin {
namespace {

constexpr uint32_t SB = kSuperTiles;  // super-block edge (tiles)

// Squared gap between two projected boxes, rounded down (so `> thr` proves
// that every pair of points drawn from the two boxes is farther apart than
// the projected threshold).  Empty boxes (lo = +inf, hi = -inf) are far from
// everything.
__device__ __forceinline__ bool boxes_far(const float* __restrict__ lo, const float* __restrict__ hi,
                                          uint64_t I, uint64_t J, uint32_t k, float thr) {
    float g2 = 0.0f;
    for (uint32_t a = 0; a < k; ++a) {
        const float l1 = lo[I * k + a], h1 = hi[I * k + a];
        const float l2 = lo[J * k + a], h2 = hi[J * k + a];
        const float gap = fmaxf(0.0f, fmaxf(__fsub_rd(l2, h1), __fsub_rd(l1, h2)));
        g2 = __fmaf_rd(gap, gap, g2);
    }
    return g2 > thr;
}

struct BoxArgs {
    const float *lo, *hi, *slo, *shi;
    uint32_t k;
    float thr;
};

// Surviving super-block pairs (SI <= SJ), appended in warp-aggregated batches.
__global__ void superpairs_kernel(uint64_t nS, BoxArgs b, uint32_t* out, unsigned long long* count) {
    const uint64_t sp = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nsp = nS * (nS + 1) / 2;
    bool keep = false;
    if (sp < nsp) {
        keep = true;
        if (b.slo) {
            uint64_t SI, SJ;
            tri_decode(sp, nS, SI, SJ);
            keep = !boxes_far(b.slo, b.shi, SI, SJ, b.k, b.thr);
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (!m) return;
    const unsigned lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) out[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)sp;
}

// One block of SB * SB / 2 threads per surviving super-block pair.  Thread
// (r, pp) tests the tile pairs (I, 2 pp') and (I, 2 pp' + 1) of row tile
// I = SI SB + r (pp' = SJ SB / 2 + pp); the up to 16 active column tiles of
// row I in this super-block (gathered from its 8 threads with two ballots)
// are paired in ascending order, and thread pp of the row emits the pp-th
// pair as one 128 x 256 block, a lone last tile with an inactive second
// half.  Entry: x = I | active mask << 30, y = Ja | (Jb - Ja) << 24 (half 0
// is column tile Ja, half 1 is Jb; Jb = Ja when half 1 is inactive).
// count[0] += blocks, count[1] += active halves (128x128 tile pairs).
constexpr uint32_t EXPAND_THREADS = SB * SB / 2;
__global__ void __launch_bounds__(EXPAND_THREADS) expand_kernel(const uint32_t* __restrict__ sps,
                                                                uint64_t nTa, uint64_t nS, BoxArgs b,
                                                                uint2* out,
                                                                unsigned long long* count) {
    __shared__ uint64_t sSI, sSJ;
    __shared__ unsigned wsum[EXPAND_THREADS / 32];
    __shared__ unsigned hsum;
    __shared__ unsigned long long sbase;
    if (threadIdx.x == 0) {
        uint64_t SI, SJ;
        tri_decode(sps[blockIdx.x], nS, SI, SJ);
        sSI = SI;
        sSJ = SJ;
        hsum = 0;
    }
    __syncthreads();
    const uint32_t pp = threadIdx.x % (SB / 2);
    const uint64_t I = sSI * SB + threadIdx.x / (SB / 2);
    const uint64_t J0 = sSJ * SB;  // first column tile of the super-block
    uint32_t mask = 0;
    for (uint32_t h = 0; h < 2; ++h) {
        const uint64_t J = J0 + 2 * pp + h;
        bool act = I < nTa && J < nTa && I <= J;
        if (act && b.lo) act = !boxes_far(b.lo, b.hi, I, J, b.k, b.thr);
        mask |= act ? (1u << h) : 0u;
    }
    // the row's active tiles: 8 lanes of the warp hold 2 bits each
    const unsigned lane = threadIdx.x & 31, wid = threadIdx.x / 32;
    const unsigned g0 = __ballot_sync(0xffffffffu, mask & 1u), g1 = __ballot_sync(0xffffffffu, mask & 2u);
    const unsigned sh = lane & ~7u;  // first lane of this row's 8
    uint32_t act16 = 0;
#pragma unroll
    for (uint32_t t = 0; t < 8; ++t)
        act16 |= (((g0 >> (sh + t)) & 1u) << (2 * t)) | (((g1 >> (sh + t)) & 1u) << (2 * t + 1));
    const uint32_t nact = __popc(act16);
    const bool keep = pp < (nact + 1) / 2;
    uint2 entry = make_uint2(0u, 0u);
    if (keep) {
        uint32_t m = act16;
        for (uint32_t k = 0; k < 2 * pp; ++k) m &= m - 1;  // drop the first 2 pp tiles
        const uint32_t ta = __ffs(m) - 1;
        m &= m - 1;
        const bool two = m != 0;
        const uint32_t tb = two ? __ffs(m) - 1 : ta;
        const uint32_t bmask = two ? 3u : 1u;
        entry = make_uint2((uint32_t)I | (bmask << 30), (uint32_t)(J0 + ta) | ((tb - ta) << 24));
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wsum[wid] = __popc(m);
    const unsigned halves = __reduce_add_sync(0xffffffffu, __popc(mask));
    if (lane == 0 && halves) atomicAdd(&hsum, halves);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned tot = 0;
        for (unsigned w = 0; w < EXPAND_THREADS / 32; ++w) {
            const unsigned c = wsum[w];
            wsum[w] = tot;
            tot += c;
        }
        sbase = tot ? atomicAdd(&count[0], (unsigned long long)tot) : 0ull;
        if (hsum) atomicAdd(&count[1], (unsigned long long)hsum);
    }
    __syncthreads();
    if (keep) out[sbase + wsum[wid] + __popc(m & ((1u << lane) - 1u))] = entry;
}

// Work list of a join of two point sets (rows: nTa tiles of A, columns: the
// pairs of B's nTb tiles), all blocks, in super-blocks of 16 row tiles x 8
// column pairs (row-major inside, super-blocks row-major) so that concurrent
// CTAs share operand rows in L2.  Closed form: every super-row but the last
// holds 16 npb entries, every super-block but the last of its super-row
// 8 qh entries (qh row tiles in the super-row).  Mask bit h: tile 2p + h < nTb.
__global__ void cross_work_kernel(uint64_t nTa, uint64_t nTb, uint64_t total, uint2* out) {
    const uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (e >= total) return;
    const uint64_t npb = (nTb + 1) / 2;
    const uint64_t SI = e / (16 * npb), rem = e - SI * 16 * npb;
    const uint64_t qh = min((uint64_t)16, nTa - SI * 16);
    const uint64_t SP = rem / (qh * 8), rem2 = rem - SP * qh * 8;
    const uint64_t pw = min((uint64_t)8, npb - SP * 8);
    const uint64_t I = SI * 16 + rem2 / pw, p = SP * 8 + rem2 % pw;
    const uint32_t mask = 1u | (2 * p + 1 < nTb ? 2u : 0u);
    out[e] = make_uint2((uint32_t)I | (mask << 30), (uint32_t)(2 * p) | (1u << 24));
}

// Band records -> pairs: a thread per record; block-level exclusive scan of
// the popcounts, one global reservation per block.
constexpr uint32_t EXPAND_BAND_THREADS = 256;
__global__ void __launch_bounds__(EXPAND_BAND_THREADS) band_expand_kernel(
    const BandRec* __restrict__ rec, uint64_t nrec, BandPair* out, uint64_t cap,
    unsigned long long* cursor) {
    using Scan = cub::BlockScan<uint32_t, EXPAND_BAND_THREADS>;
    __shared__ typename Scan::TempStorage tmp;
    __shared__ unsigned long long sbase;
    const uint64_t e = blockIdx.x * (uint64_t)EXPAND_BAND_THREADS + threadIdx.x;
    BandRec r{0, 0, 0, 0};
    if (e < nrec) r = rec[e];
    const uint32_t cnt = __popc(r.mask);
    uint32_t off = 0, total = 0;
    Scan(tmp).ExclusiveSum(cnt, off, total);
    if (threadIdx.x == 0) sbase = total ? atomicAdd(cursor, (unsigned long long)total) : 0ull;
    __syncthreads();
    uint64_t o = sbase + off;
    uint32_t m = r.mask;
    const uint32_t flag = r.j0 & kBandBoth, j0 = r.j0 & ~kBandBoth;
    while (m) {
        const uint32_t c = __ffs(m) - 1;
        m &= m - 1;
        if (o < cap) out[o] = BandPair{r.i, (j0 + c) | flag};
        ++o;
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

// Builds the list of surviving blocks: super-block pairs first (one thread
// each), then the blocks of the survivors (one thread block each).  nT: row
// tiles (even); nTa: tiles holding data rows.
int build_worklist(uint64_t nT, uint64_t nTa, const LearnedBoxes* boxes, float thr,
                   DBuf<uint2>& work, uint64_t* nwork_out, uint64_t* ntiles_out, cudaStream_t s) {
    *nwork_out = 0;
    *ntiles_out = 0;
    if (nT == 0) return EJOIN_OK;
    if (nT % 2 || nTa > nT) return set_error(EJOIN_EINTERNAL, "work list: odd tile count");
    const uint64_t nS = (nT + SB - 1) / SB;
    const uint64_t nsp = nS * (nS + 1) / 2;
    if (nsp > 0xffffffffull) return set_error(EJOIN_EUNSUPPORTED, "work list too large");
    BoxArgs b{nullptr, nullptr, nullptr, nullptr, 0, thr};
    if (boxes) b = BoxArgs{boxes->lo.p, boxes->hi.p, boxes->slo.p, boxes->shi.p, boxes->k, thr};
    DBuf<uint32_t> sps;
    DBuf<unsigned long long> cnt;
    EJ_TRY(sps.alloc(nsp, s, "super-block pairs"));
    EJ_TRY(cnt.alloc(3, s, "work-list counters"));
    EJ_TRY(cnt.zero(s));
    superpairs_kernel<<<(unsigned)((nsp + 255) / 256), 256, 0, s>>>(nS, b, sps.p, cnt.p);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    unsigned long long nkeep = 0;
    EJ_CUDA(cudaMemcpyAsync(&nkeep, cnt.p, sizeof nkeep, cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    EJ_TRY(work.alloc(nkeep ? nkeep * EXPAND_THREADS : 1, s, "work list"));
    if (nkeep) {
        if (nkeep > 0x7fffffffull) return set_error(EJOIN_EUNSUPPORTED, "work list too large");
        // back into triangular (row-major) order: consecutive work then shares row blocks
        DBuf<uint32_t> sorted;
        EJ_TRY(sorted.alloc(nkeep, s, "sorted super-block pairs"));
        size_t tb = 0;
        EJ_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tb, sps.p, sorted.p, (int)nkeep, 0, 32, s));
        DBuf<uint8_t> tmp;
        EJ_TRY(tmp.alloc(tb, s, "sort scratch"));
        EJ_CUDA(cub::DeviceRadixSort::SortKeys(tmp.p, tb, sps.p, sorted.p, (int)nkeep, 0, 32, s));
        note_launch(4);
        expand_kernel<<<(unsigned)nkeep, EXPAND_THREADS, 0, s>>>(sorted.p, nTa, nS, b, work.p,
                                                                 cnt.p + 1);
        EJ_CUDA(cudaGetLastError());
        note_launch();
    }
    unsigned long long tot[2] = {0, 0};
    EJ_CUDA(cudaMemcpyAsync(tot, cnt.p + 1, sizeof tot, cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    *nwork_out = tot[0];
    *ntiles_out = tot[1];
    return EJOIN_OK;
}

int launch_band_expand(const BandRec* rec, uint64_t nrec, BandPair* out, uint64_t cap,
                       cudaStream_t s) {
    if (nrec == 0) return EJOIN_OK;
    DBuf<unsigned long long> cur;
    EJ_TRY(cur.alloc(1, s, "band cursor"));
    EJ_TRY(cur.zero(s));
    band_expand_kernel<<<(unsigned)((nrec + EXPAND_BAND_THREADS - 1) / EXPAND_BAND_THREADS),
                         EXPAND_BAND_THREADS, 0, s>>>(rec, nrec, out, cap, cur.p);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

int build_worklist_cross(uint64_t nTa, uint64_t nTb, DBuf<uint2>& work, uint64_t* nwork_out,
                         uint64_t* ntiles_out, cudaStream_t s) {
    const uint64_t total = nTa * ((nTb + 1) / 2);
    *nwork_out = total;
    *ntiles_out = nTa * nTb;
    if (total == 0) return EJOIN_OK;
    EJ_TRY(work.alloc(total, s, "work list"));
    cross_work_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(nTa, nTb, total, work.p);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

// Every stride-th entry of a work list (a systematic sample of its blocks).
__global__ void sample_work_kernel(const uint2* __restrict__ work, uint64_t nsample,
                                   uint64_t stride, uint2* __restrict__ out) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < nsample) out[i] = work[i * stride];
}

int sample_worklist(const uint2* work, uint64_t nwork, uint64_t stride, DBuf<uint2>& out,
                    uint64_t* nsample_out, cudaStream_t s) {
    const uint64_t ns = stride ? (nwork + stride - 1) / stride : 0;
    *nsample_out = ns;
    if (ns == 0) return EJOIN_OK;
    EJ_TRY(out.alloc(ns, s, "sampled work list"));
    sample_work_kernel<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(work, ns, stride, out.p);
    EJ_CUDA(cudaGetLastError());
    note_launch();
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
