// k_lists.cu -- neighbour lists (CSR) of the exact self join.
//
// The reference returns only the total (gpu_join.cu:210-322); its result-set
// kernels (kernel_join.cu:139-162) are dead code.  Here the lists come from a
// second pass of the same exact join that emits its neighbour pairs: the
// tensor-core screen appends one in-record per row and 32-column chunk with
// certain neighbours, the band recheck and the FP64 arbiter append single
// pairs.  Every neighbour pair is emitted exactly once (the screens visit
// each unordered pair once; kBandBoth marks pairs that credit both points),
// so the per-point counts of the counting pass give the CSR offsets, and a
// scatter through per-point cursors fills the lists; a check then requires
// every cursor to end exactly at the next point's offset, and a segmented
// sort puts every list in ascending order (deterministic output).
#include <cub/cub.cuh>

#include "ejoin_internal.cuh"

namespace ejoin {
namespace {

__global__ void widen_kernel(const int32_t* __restrict__ c, uint64_t n, unsigned long long* out) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint32_t)c[i];
}

__device__ __forceinline__ void put(unsigned long long* cur, uint32_t* nb, uint64_t total,
                                    uint32_t at, uint32_t value, unsigned* err) {
    const unsigned long long slot = atomicAdd(&cur[at], 1ull);
    if (slot < total) nb[slot] = value;
    else atomicOr(err, 1u);
}

// in-records: the pairs (i, j0 + c) for the set bits c (packed indices)
__global__ void scatter_in_kernel(const BandRec* __restrict__ rec, uint64_t nrec,
                                  const uint32_t* __restrict__ perm, uint64_t n,
                                  unsigned long long* cur, uint32_t* nb, uint64_t total,
                                  unsigned* err) {
    const uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (e >= nrec) return;
    const BandRec r = rec[e];
    const uint32_t j0 = r.j0 & ~kBandBoth;
    const bool both = (r.j0 & kBandBoth) != 0;
    if (r.i >= n) {
        atomicOr(err, 2u);
        return;
    }
    const uint32_t oi = perm ? perm[r.i] : r.i;
    uint32_t m = r.mask;
    while (m) {
        const uint32_t c = __ffs(m) - 1;
        m &= m - 1;
        const uint32_t j = j0 + c;
        if (j >= n) {
            atomicOr(err, 2u);
            continue;
        }
        const uint32_t oj = perm ? perm[j] : j;
        put(cur, nb, total, oi, oj, err);
        if (both) put(cur, nb, total, oj, oi, err);
    }
}

// single pairs (i, j | both) (packed indices)
__global__ void scatter_pairs_kernel(const BandPair* __restrict__ pq, uint64_t np,
                                     const uint32_t* __restrict__ perm, uint64_t n,
                                     unsigned long long* cur, uint32_t* nb, uint64_t total,
                                     unsigned* err) {
    const uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    const BandPair p = pq[e];
    const uint32_t i = p.i, j = p.j & ~kBandBoth;
    if (i >= n || j >= n) {
        atomicOr(err, 2u);
        return;
    }
    const uint32_t oi = perm ? perm[i] : i, oj = perm ? perm[j] : j;
    put(cur, nb, total, oi, oj, err);
    if (p.j & kBandBoth) put(cur, nb, total, oj, oi, err);
}

__global__ void check_cursor_kernel(const unsigned long long* __restrict__ cur,
                                    const unsigned long long* __restrict__ off, uint64_t n,
                                    unsigned* err) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n && cur[i] != off[i + 1]) atomicOr(err, 4u);
}

}  // namespace

int csr_offsets(const int32_t* counts, uint64_t n, uint64_t total, unsigned long long* offsets,
                cudaStream_t s) {
    if (n > 0x7fffffffull) return set_error(EJOIN_EUNSUPPORTED, "neighbour lists: too many points");
    if (n) {
        DBuf<unsigned long long> w;
        EJ_TRY(w.alloc(n, s, "list lengths"));
        widen_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(counts, n, w.p);
        EJ_CUDA(cudaGetLastError());
        size_t tb = 0;
        EJ_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, w.p, offsets, (int)n, s));
        DBuf<uint8_t> tmp;
        EJ_TRY(tmp.alloc(tb, s, "scan scratch"));
        EJ_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, w.p, offsets, (int)n, s));
        note_launch(2);
    }
    const unsigned long long t = total;
    EJ_CUDA(cudaMemcpyAsync(offsets + n, &t, sizeof t, cudaMemcpyHostToDevice, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    return EJOIN_OK;
}

int csr_fill(const unsigned long long* offsets, uint64_t n, uint64_t total, const BandRec* inq,
             uint64_t nin, const BandPair* pq, uint64_t np, const uint32_t* perm, uint32_t* nb,
             cudaStream_t s) {
    if (total > 0x7fffffffull)
        return set_error(EJOIN_EUNSUPPORTED, "neighbour lists: %llu pairs exceed 2^31 - 1",
                         (unsigned long long)total);
    if (total == 0) return EJOIN_OK;
    DBuf<unsigned long long> cur;
    DBuf<uint32_t> raw;
    DBuf<unsigned> err;
    EJ_TRY(cur.alloc(n, s, "list cursors"));
    EJ_TRY(raw.alloc(total, s, "unsorted lists"));
    EJ_TRY(err.alloc(1, s, "list check"));
    EJ_TRY(err.zero(s));
    EJ_CUDA(cudaMemcpyAsync(cur.p, offsets, n * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s));
    if (nin)
        scatter_in_kernel<<<(unsigned)((nin + 255) / 256), 256, 0, s>>>(inq, nin, perm, n, cur.p,
                                                                        raw.p, total, err.p);
    if (np)
        scatter_pairs_kernel<<<(unsigned)((np + 255) / 256), 256, 0, s>>>(pq, np, perm, n, cur.p,
                                                                          raw.p, total, err.p);
    check_cursor_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(cur.p, offsets, n, err.p);
    EJ_CUDA(cudaGetLastError());
    note_launch(3);
    unsigned h = 0;
    EJ_CUDA(cudaMemcpyAsync(&h, err.p, sizeof h, cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    if (h) return set_error(EJOIN_EINTERNAL, "neighbour lists: emitted pairs disagree with the counts (%u)", h);
    size_t tb = 0;
    EJ_CUDA(cub::DeviceSegmentedSort::SortKeys(nullptr, tb, raw.p, nb, (int)total, (int)n, offsets,
                                               offsets + 1, s));
    DBuf<uint8_t> tmp;
    EJ_TRY(tmp.alloc(tb, s, "sort scratch"));
    EJ_CUDA(cub::DeviceSegmentedSort::SortKeys(tmp.p, tb, raw.p, nb, (int)total, (int)n, offsets,
                                               offsets + 1, s));
    note_launch(2);
    return EJOIN_OK;
}

}  // namespace ejoin
