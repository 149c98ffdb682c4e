// k_umma.cu -- the tcgen05 Gram screen (EJOIN_BF16 / BF16_SPLIT / FP16 / FP8_E4M3).
//
// Re-designs the reference's main tensor path,
// distanceCalculationBruteForceTensorHalf (kernel_join.cu:328-524): there a
// warp computes -2*Q*C^T + |c|^2 for 16 queries x 16 candidates per wmma
// m16n16k16, round-trips every k-chunk through shared memory, re-adds the
// query norms in scalar code and bumps one global counter per hit with
// sqrt(|d2|) <= eps.  Here:
//
//  * A persistent CTA per SM walks a list of blocks of 128 rows (row tile I)
//    x 256 columns (two column tiles Ja, Jb, not necessarily adjacent: the
//    B slab is loaded as two 128-row boxes), taking runs of consecutive list
//    entries.  Each 128x128 half carries an "active" bit: it lies in the
//    upper triangle (J >= I) and was not pruned; an inactive half (a row's
//    odd last tile) is computed but ignored.  N = 256 per MMA instruction: on
//    GB300 a tcgen05.mma of 128x256x16 takes about as long to issue and
//    retire as one of 128x128x16 (measured: 1.8 vs 0.92 PFLOP/s through the
//    same TMA / MMA pipeline), so the wide tile doubles the tensor-pipe
//    throughput, and pairing lone tiles halves their cost.
//  * Warp 0 streams the K-slabs of both blocks into a 4-stage ring with TMA
//    (128-byte swizzle; a 128-row A slab and a 256-row B slab per stage; the
//    aug boxes of a block go to a separate 2-slot ring).  Four stages in
//    flight are what the hi+lo MMA sequence needs to reach the tensor-pipe
//    peak (measured: 1.77 PFLOP/s with 4, 1.33 with 3).
//    One thread of warp 1 issues tcgen05.mma (M=128, N=256, K=16 per
//    instruction) into one of two FP32 accumulators of 256 tensor-memory
//    columns each, so the next block's MMAs run while 16 epilogue warps read
//    the previous one.
//  * Operand rows are [hi | lo] (k_prep.cu) with a separate 16-element aug
//    row (32-byte swizzle).  With the hi+lo split the MMAs form hi*hi + hi*lo
//    + lo*hi.  The aug MMA adds -alpha_i - alpha_j, so the accumulator holds
//    C_ij = q_i.q_j - alpha_i - alpha_j and the rigorous screen is a sign test:
//        C >= 0          pair certainly within eps        (counted)
//        C < -W_iK       pair certainly outside eps
//        otherwise       band: queued for the FP64 recheck
//    W_iK = beta_i + max beta over the 32-column chunk K >= beta_i + beta_j
//    (one value per row and column chunk, so the test costs one add per
//    element, like a tile-wide width, with a narrower band).
//  * Each epilogue warp reads its two 32x32 chunks one after the other with
//    tcgen05.ld.red (the load also returns each lane's maximum, which decides
//    the all-out fast path), packs sign bits with one funnel shift per
//    element, counts rows with popc, transposes 32x32 bit blocks across the
//    warp to count columns (off-diagonal tiles credit both points), and a
//    flusher warp adds the per-block counts to global memory.  A block's
//    counting comes before the wait for the next block's accumulator.  No
//    distance reaches global memory.
//
// Every wait is bounded (umma_ptx.cuh); on expiry all roles stop, in-flight
// copies and MMAs are drained (bounded) and tensor memory is freed.
#include "tmap.cuh"
#include "umma_ptx.cuh"

namespace ejoin {
namespace {

constexpr int SLAB_A = 128 * 128;  // 128 rows x 128 bytes
constexpr int SLAB_B = 256 * 128;  // 256 rows x 128 bytes
constexpr int AUG_A = 128 * 32;    // 128 rows x 32 bytes (16 elements)
constexpr int AUG_B = 256 * 32;
// stage: A slab | B slab; aug slot: A aug | B aug (one per block); every part
// starts on a 1024-byte boundary
constexpr int STAGE_BYTES = SLAB_A + SLAB_B;
constexpr int NST = 4;
constexpr int AUG_SLOT = AUG_A + AUG_B;
constexpr int NAUG = 2;
constexpr uint32_t DATA_TX = SLAB_A + SLAB_B;
constexpr int NUM_EPI_WARPS = 16;          // 4 per SM sub-partition (latency hiding)
constexpr int FLUSH_WARP = 2 + NUM_EPI_WARPS;  // adds the per-block counts to global memory
constexpr int NTHREADS = (3 + NUM_EPI_WARPS) * 32;
constexpr uint32_t ACC_COLS = 256;         // one 128x256 FP32 accumulator
constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;
constexpr uint32_t FULL = 0xffffffffu;

// Work-list entry: x = row tile I | active mask << 30, y = Ja | (Jb - Ja) << 24:
// half 0 of the block is column tile Ja, half 1 is Jb (bit h of the mask:
// half h is computed).
constexpr uint32_t kRowMask = (1u << 30) - 1u;
__device__ __forceinline__ uint32_t e_row(uint2 e) { return e.x & kRowMask; }
__device__ __forceinline__ uint32_t e_mask(uint2 e) { return e.x >> 30; }
__device__ __forceinline__ uint32_t e_col(uint2 e, uint32_t h) {
    const uint32_t ja = e.y & 0xffffffu;
    return h ? ja + ((e.y >> 24) & 63u) : ja;
}

struct GramArgs {
    const uint2* work;
    uint64_t nwork;
    const float* cmax;  // per 32-row chunk of B: max beta
    const float* beta;  // per row: beta (out margin, Gram units)
    const float* tsig;  // FP8: per-tile minimum row scale (null for 16-bit operands)
    const float* sig;   // FP8: per-row scale
    int32_t* counts;
    BandRec* band;
    uint64_t band_cap;
    DevStatus* st;
    uint32_t nhi;    // data slabs (128-byte rows) per part
    uint32_t split;  // hi + lo
    uint32_t fmt;    // 16-bit operands: 0 = FP16, 1 = BF16 (instruction-descriptor format)
    uint32_t lrun;   // log2 of the run length: entries a CTA takes consecutively
    uint32_t cross;  // rows of A against a different set B: count rows only
    Emit em;         // neighbour-list emission (em.cnt null: counts only)
};

__device__ __forceinline__ uint2 entry_or_end(const GramArgs& a, uint64_t u) {
    return u < a.nwork ? __ldg(&a.work[u]) : make_uint2(0xffffffffu, 0xffffffffu);
}

// Entry idx (0, 1, 2, ...) of this CTA's sequence: runs of 2^lrun consecutive
// work-list entries, runs dealt round-robin over the CTAs (so the CTAs
// running at the same time stay within a window of the list that shares
// operand rows in L2).  Increasing in idx.
__device__ __forceinline__ uint64_t item_at(uint64_t idx, uint32_t lrun) {
    const uint64_t k = idx >> lrun, r = idx & ((1ull << lrun) - 1ull);
    return ((k * gridDim.x + blockIdx.x) << lrun) + r;
}

constexpr uint32_t BAND_SMEM = 192;   // staged band records per count buffer

struct Ctl {
    uint64_t full[NST], empty[NST];
    uint64_t gfull[NAUG], gempty[NAUG];  // aug slots
    uint64_t tfull[2], tempty[2];
    uint64_t ebar[2];   // epilogue warps done with the counts of buffer b
    uint64_t fdone[2];  // flusher done with (and cleared) the counts of buffer b
    uint64_t fin;
    uint32_t tmem_base;
    int rowacc[2][128];
    int colacc[2][256];
    uint32_t band_n[2];                  // band entries staged for buffer b
    uint32_t has_counts[2];              // some epilogue warp added counts to buffer b
    BandRec band_buf[2][BAND_SMEM];      // staged band records (flushed by the flusher warp)
};

constexpr size_t RING_BYTES = (size_t)NST * STAGE_BYTES + (size_t)NAUG * AUG_SLOT;
constexpr size_t SMEM_BYTES = 1024 + RING_BYTES + sizeof(Ctl);
static_assert(SMEM_BYTES <= 232448, "shared memory budget");

// 32x32 bit-matrix transpose across the warp: lane r holds row r (bit c =
// column c); afterwards lane c holds column c (bit r = row r).
__device__ __forceinline__ uint32_t transpose32(uint32_t x, uint32_t lane) {
    const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
    uint32_t j = 16;
#pragma unroll
    for (int l = 0; l < 5; ++l, j >>= 1) {
        const uint32_t m = masks[l];
        const uint32_t y = __shfl_xor_sync(FULL, x, j);
        x = (lane & j) ? (((y >> j) & m) | (x & ~m)) : ((x & m) | ((y & m) << j));
    }
    return x;
}

// Element offset of K-slab `step` of a block: [hi0, lo0, hi1, lo1, ...] with
// the split, [hi0, hi1, ...] without.
template <int OPK>
__device__ __forceinline__ uint32_t slab_x(uint32_t step, uint32_t nhi, uint32_t split) {
    constexpr uint32_t E = OPK ? 128u : 64u;  // elements per 128-byte slab row
    if (split) return (step & 1) ? E * nhi + E * (step >> 1) : E * (step >> 1);
    return E * step;
}

// Column counts of one 32 x 32 in-mask (lane = row): sparse masks (at most
// 3 bits per lane) add per bit to shared memory, denser ones transpose the
// bit block across the warp and add one count per column.
__device__ __forceinline__ void col_counts(uint32_t inm, int* cacc, uint32_t lane) {
    const uint32_t mp = __reduce_max_sync(FULL, __popc(inm));
    if (mp == 0) return;
    if (mp <= 3) {
        uint32_t m = inm;
        while (m) {
            const uint32_t c = __ffs(m) - 1;
            m &= m - 1;
            atomicAdd(&cacc[c], 1);
        }
    } else {
        const int cc = __popc(transpose32(inm, lane));
        if (cc) atomicAdd(&cacc[lane], cc);
    }
}

// In / band bit masks of one 32 x 32 chunk (lane = row, v[c] = column c; mx
// = the lane's maximum, reduced by the tensor-memory load).
// Fast path: if max + W < 0 over the chunk, every pair in it is certainly out
// (rounding of the FP32 add is monotone, so max + W >= 0 whenever any
// element is >= -W).
__device__ __forceinline__ bool classify(const uint32_t (&v)[32], float mx, float W,
                                         uint32_t& inm, uint32_t& bandm) {
    inm = bandm = 0;
    if (!__any_sync(FULL, mx + W >= 0.0f)) return false;
    // sign bits, four independent 8-column chains
    uint32_t ng[4] = {0, 0, 0, 0}, nw[4] = {0, 0, 0, 0};
#pragma unroll
    for (int c = 7; c >= 0; --c)
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            const uint32_t x = v[8 * g + c];
            ng[g] = __funnelshift_l(x, ng[g], 1);
            nw[g] = __funnelshift_l(__float_as_uint(__uint_as_float(x) + W), nw[g], 1);
        }
    const uint32_t neg = ng[0] | (ng[1] << 8) | (ng[2] << 16) | (ng[3] << 24);
    const uint32_t negw = nw[0] | (nw[1] << 8) | (nw[2] << 16) | (nw[3] << 24);
    inm = ~neg;
    bandm = neg & ~negw;
    return true;
}

// Band records of the two chunks of a warp: a lane with band pairs in a chunk
// writes one record (its row, the chunk's first column, the bit mask).  Slots
// come from one shared-memory reservation per warp (ranks from ballots);
// records beyond the staging area go to global memory directly.
__device__ __forceinline__ void stage_band(const GramArgs& a, Ctl& S, uint32_t b, uint32_t bd0,
                                           uint32_t bd1, uint32_t row, uint32_t col0, bool diag,
                                           uint32_t lane) {
    const uint32_t b0 = __ballot_sync(FULL, bd0 != 0), b1 = __ballot_sync(FULL, bd1 != 0);
    const uint32_t n0 = __popc(b0);
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&S.band_n[b], n0 + __popc(b1));
    base = __shfl_sync(FULL, base, 0);
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t flag = diag ? 0u : kBandBoth;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const uint32_t m = k ? bd1 : bd0;
        if (!m) continue;
        const uint32_t slot = base + (k ? n0 + __popc(b1 & lt) : __popc(b0 & lt));
        const BandRec r{row, (col0 + 32u * k) | flag, m, 0u};
        if (slot < BAND_SMEM) {
            S.band_buf[b][slot] = r;
        } else {
            const unsigned long long g = atomicAdd(&a.st->band_count, 1ull);
            atomicAdd(&a.st->band_pairs, (unsigned long long)__popc(m));
            atomicAdd(&a.st->band_records, 1ull);
            if (g < a.band_cap) a.band[g] = r;
        }
    }
}

// In-records of the two chunks of a warp (neighbour lists): a lane with
// in-pairs in a chunk appends (row, first column | both, mask); one global
// reservation per warp.
__device__ __forceinline__ void emit_in(const GramArgs& a, uint32_t in0, uint32_t in1,
                                        uint32_t row, uint32_t col0, bool diag, uint32_t lane) {
    const uint32_t b0 = __ballot_sync(FULL, in0 != 0), b1 = __ballot_sync(FULL, in1 != 0);
    const uint32_t n0 = __popc(b0), tot = n0 + __popc(b1);
    if (!tot) return;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&a.em.cnt[0], (unsigned long long)tot);
    base = __shfl_sync(FULL, base, 0);
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t flag = diag ? 0u : kBandBoth;
    if (in0) {
        const unsigned long long slot = base + __popc(b0 & lt);
        if (slot < a.em.inq_cap) a.em.inq[slot] = BandRec{row, col0 | flag, in0, 0u};
    }
    if (in1) {
        const unsigned long long slot = base + n0 + __popc(b1 & lt);
        if (slot < a.em.inq_cap) a.em.inq[slot] = BandRec{row, (col0 + 32u) | flag, in1, 0u};
    }
}

// OPK 0: 16-bit operands, data MMAs kind::f16; OPK 1: E4M3 operands, data
// MMAs kind::f8f6f4 (K = 32 per instruction, same 32-byte k-steps), the aug
// MMA stays kind::f16 in BF16 and accumulates into the same tensor memory.
template <int OPK>
__global__ void __launch_bounds__(NTHREADS, 1)
    gram_kernel(const __grid_constant__ CUtensorMap tqa, const __grid_constant__ CUtensorMap tqb,
                const __grid_constant__ CUtensorMap taa, const __grid_constant__ CUtensorMap tab,
                const GramArgs a) {
    extern __shared__ uint8_t smraw[];
    uint8_t* stages = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
    uint8_t* augs = stages + (size_t)NST * STAGE_BYTES;
    Ctl& S = *reinterpret_cast<Ctl*>(stages + RING_BYTES);
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x & 31;

    if (warp == 1) {
        ptx::tmem_alloc(&S.tmem_base, TMEM_COLS);
        ptx::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            ptx::mbar_init(&S.full[s], 1);
            ptx::mbar_init(&S.empty[s], 1);
        }
        for (int g = 0; g < NAUG; ++g) {
            ptx::mbar_init(&S.gfull[g], 1);
            ptx::mbar_init(&S.gempty[g], 1);
        }
        for (int b = 0; b < 2; ++b) {
            ptx::mbar_init(&S.tfull[b], 1);
            ptx::mbar_init(&S.tempty[b], NUM_EPI_WARPS);
            ptx::mbar_init(&S.ebar[b], NUM_EPI_WARPS);
            ptx::mbar_init(&S.fdone[b], 1);
        }
        ptx::mbar_init(&S.fin, 1);
        ptx::fence_barrier_init();
        ptx::tma_prefetch_desc(&tqa);
        ptx::tma_prefetch_desc(&tqb);
        ptx::tma_prefetch_desc(&taa);
        ptx::tma_prefetch_desc(&tab);
    }
    for (int i = threadIdx.x; i < 2 * (128 + 256); i += NTHREADS) {
        if (i < 256) (&S.rowacc[0][0])[i] = 0;
        else (&S.colacc[0][0])[i - 256] = 0;
    }
    if (threadIdx.x < 2) {
        S.band_n[threadIdx.x] = 0;
        S.has_counts[threadIdx.x] = 0;
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t nsteps = a.nhi * (a.split ? 2u : 1u);

    if (warp == 0) {
        // ------------------------------------------------ TMA producer
        if (lane == 0) {
            uint32_t st = 0, ph = 0;
            uint32_t issued_ph[NST];
            uint32_t issued = 0;
            uint32_t aug_ph[NAUG] = {0, 0};
            uint64_t aug_issued = 0;
            bool ok = true;
            // test hook (DevStatus::withhold): the first stage is never
            // issued, so the waits on it expire; it is not counted in
            // `issued` and the producer stops before stage 0 comes round
            // again, so the drain below never waits for it
            bool withhold = *(volatile unsigned*)&a.st->withhold != 0u;
            // entries are read one block ahead (their latency hides behind a block)
            uint2 wnext = entry_or_end(a, item_at(0, a.lrun));
            for (uint64_t idx = 0; ok; ++idx) {
                const uint64_t u = item_at(idx, a.lrun);
                if (u >= a.nwork) break;
                const uint2 w = wnext;
                wnext = entry_or_end(a, item_at(idx + 1, a.lrun));
                const int32_t ya = (int32_t)(e_row(w) * 128u);
                const int32_t yb0 = (int32_t)(e_col(w, 0) * 128u), yb1 = (int32_t)(e_col(w, 1) * 128u);
                {
                    // this block's aug boxes
                    const uint32_t g = (uint32_t)(idx % NAUG), guse = (uint32_t)(idx / NAUG);
                    if (!ptx::mbar_wait(&S.gempty[g], (guse & 1u) ^ 1u, a.st, 11)) break;
                    uint8_t* sg = augs + (size_t)g * AUG_SLOT;
                    ptx::mbar_arrive_expect_tx(&S.gfull[g], AUG_SLOT);
                    ptx::tma_load_2d(sg, &taa, 0, ya, &S.gfull[g]);
                    ptx::tma_load_2d(sg + AUG_A, &tab, 16, yb0, &S.gfull[g]);
                    ptx::tma_load_2d(sg + AUG_A + AUG_B / 2, &tab, 16, yb1, &S.gfull[g]);
                    aug_ph[g] = guse & 1u;
                    ++aug_issued;
                }
                for (uint32_t step = 0; step < nsteps; ++step) {
                    if (!ptx::mbar_wait(&S.empty[st], ph ^ 1u, a.st, 10)) {
                        ok = false;
                        break;
                    }
                    uint8_t* sa = stages + (size_t)st * STAGE_BYTES;
                    const int32_t x = (int32_t)slab_x<OPK>(step, a.nhi, a.split);
                    if (withhold) {
                        withhold = false;
                    } else {
                        ptx::mbar_arrive_expect_tx(&S.full[st], DATA_TX);
                        ptx::tma_load_2d(sa, &tqa, x, ya, &S.full[st]);
                        ptx::tma_load_2d(sa + SLAB_A, &tqb, x, yb0, &S.full[st]);
                        ptx::tma_load_2d(sa + SLAB_A + SLAB_B / 2, &tqb, x, yb1, &S.full[st]);
                        issued_ph[st] = ph;
                        ++issued;
                    }
                    if (++st == NST) {
                        st = 0;
                        ph ^= 1u;
                    }
                }
            }
            // drain: every issued copy has landed before the CTA can exit
            const uint32_t last = issued < (uint32_t)NST ? issued : (uint32_t)NST;
            for (uint32_t k = 0; k < last; ++k) {
                const uint32_t s = (st + NST - 1 - k) % NST;
                ptx::mbar_wait_drain(&S.full[s], issued_ph[s]);
            }
            for (uint32_t g = 0; g < NAUG; ++g)
                if (aug_issued > g) ptx::mbar_wait_drain(&S.gfull[g], aug_ph[g]);
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = OPK ? ptx::idesc_f32acc(0, 0, 128, ACC_COLS)
                                       : ptx::idesc_f32acc(a.fmt, a.fmt, 128, ACC_COLS);
            const uint32_t idesc_aug = OPK ? ptx::idesc_f32acc(1, 1, 128, ACC_COLS) : idesc;
            auto mma = [&](uint32_t d, uint64_t ad, uint64_t bd, uint32_t acc_) {
                if (OPK) ptx::mma_f8(d, ad, bd, idesc, acc_);
                else ptx::mma_f16(d, ad, bd, idesc, acc_);
            };
            uint32_t st = 0, ph = 0, it = 0;
            bool ok = true;
            auto take = [&](uint32_t& s_out) -> bool {
                if (!ptx::mbar_wait(&S.full[st], ph, a.st, 20)) return false;
                s_out = st;
                if (++st == NST) {
                    st = 0;
                    ph ^= 1u;
                }
                return true;
            };
            for (uint64_t idx = 0; ok; ++idx, ++it) {
                if (item_at(idx, a.lrun) >= a.nwork) break;
                const uint32_t b = it & 1u, use = it >> 1;
                if (!ptx::mbar_wait(&S.tempty[b], (use & 1u) ^ 1u, a.st, 21)) break;
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem + b * ACC_COLS;
                // Order by magnitude (the accumulation bound of screen_params
                // in api.cu relies on it): the first slab's hi*lo and lo*hi
                // products, then the hi*hi ones, then the later slabs, and
                // the aug step (-alpha_i - alpha_j) last.
                uint32_t acc = 0;
                for (uint32_t c = 0; c < a.nhi && ok; ++c) {
                    uint32_t s_hi, s_lo = 0;
                    if (!take(s_hi)) { ok = false; break; }
                    if (a.split && !take(s_lo)) { ok = false; break; }
                    ptx::tc_fence_after();
                    uint8_t* st_hi = stages + (size_t)s_hi * STAGE_BYTES;
                    const uint64_t ah = ptx::sdesc_sw128(ptx::smem_u32(st_hi));
                    const uint64_t bh = ptx::sdesc_sw128(ptx::smem_u32(st_hi + SLAB_A));
                    if (a.split) {
                        uint8_t* st_lo = stages + (size_t)s_lo * STAGE_BYTES;
                        const uint64_t al = ptx::sdesc_sw128(ptx::smem_u32(st_lo));
                        const uint64_t bl = ptx::sdesc_sw128(ptx::smem_u32(st_lo + SLAB_A));
#pragma unroll
                        for (uint32_t kk = 0; kk < 4; ++kk) {
                            mma(d_tmem, ah + 2 * kk, bl + 2 * kk, acc);
                            mma(d_tmem, al + 2 * kk, bh + 2 * kk, 1);
                            acc = 1;
                        }
#pragma unroll
                        for (uint32_t kk = 0; kk < 4; ++kk) mma(d_tmem, ah + 2 * kk, bh + 2 * kk, 1);
                        ptx::mma_commit(&S.empty[s_hi]);
                        ptx::mma_commit(&S.empty[s_lo]);
                    } else {
#pragma unroll
                        for (uint32_t kk = 0; kk < 4; ++kk) {
                            mma(d_tmem, ah + 2 * kk, bh + 2 * kk, acc);
                            acc = 1;
                        }
                        ptx::mma_commit(&S.empty[s_hi]);
                    }
                }
                if (!ok) break;
                {
                    // aug: A side (alpha_i, -1) x B side (-1, alpha_j), one K = 16 step
                    const uint32_t g = (uint32_t)(idx % NAUG), guse = (uint32_t)(idx / NAUG);
                    if (!ptx::mbar_wait(&S.gfull[g], guse & 1u, a.st, 22)) break;
                    ptx::tc_fence_after();
                    uint8_t* sg = augs + (size_t)g * AUG_SLOT;
                    ptx::mma_f16(d_tmem, ptx::sdesc_sw32(ptx::smem_u32(sg)),
                                 ptx::sdesc_sw32(ptx::smem_u32(sg + AUG_A)), idesc_aug, acc);
                    ptx::mma_commit(&S.gempty[g]);
                }
                ptx::mma_commit(&S.tfull[b]);
            }
            // drain: all MMAs complete before tensor memory is freed
            ptx::mma_commit(&S.fin);
            ptx::mbar_wait_drain(&S.fin, 0);
        }
    } else if (warp < FLUSH_WARP) {
        // ------------------------------------------------ epilogue warps
        // warp e reads lane quarter (warp % 4) and the 64 columns 64 * (e / 4),
        // which lie in half h = e / 8 (column tile Ja or Jb)
        const uint32_t ew = warp - 2;          // 0..15
        const uint32_t q = warp & 3u;          // tensor-memory lane quarter
        const uint32_t cg = ew >> 2;           // 64-column group
        const uint32_t h = cg >> 1;            // half
        uint32_t it = 0;
        // band width of row i against a 32-column chunk K of column tile J:
        // W >= beta_i + max beta over K >= beta_i + beta_j for every j in K
        // (Gram units; FP8 operands: divided by sigma_i sigma_J,min, the
        // accumulator's unit for pair (i, j) being 1 / (sigma_i sigma_j)); the
        // sum is rounded up by the 2^-20 relative margin, division by the
        // power-of-two scales is exact.  0 for an inactive half.
        // Latency: entries are read two blocks ahead and the raw margins one
        // block ahead, both consumed a block later, so no global-load latency
        // lands on a block's own path.
        struct Margins {
            float b, t0, t1, sr, st;
            bool on;
        };
        auto load_margins = [&](uint2 e) -> Margins {
            Margins m{0.0f, 0.0f, 0.0f, 1.0f, 1.0f, false};
            if (e.x != 0xffffffffu && ((e_mask(e) >> h) & 1u)) {
                const uint32_t Je = e_col(e, h);
                const uint32_t r = e_row(e) * 128u + q * 32u + lane;
                const uint32_t c = (Je * 128u + (cg & 1u) * 64u) / 32u;  // first chunk
                m.b = __ldg(&a.beta[r]);
                m.t0 = __ldg(&a.cmax[c]);
                m.t1 = __ldg(&a.cmax[c + 1]);
                if (OPK) {
                    m.sr = __ldg(&a.sig[r]);
                    m.st = __ldg(&a.tsig[Je]);
                }
                m.on = true;
            }
            return m;
        };
        // chunk k (0, 1) of the warp's 64 columns: W >= beta_i + max beta over
        // the chunk's 32 columns
        auto width = [&](const Margins& m, int k) -> float {
            if (!m.on) return 0.0f;
            const float sm = m.b + (k ? m.t1 : m.t0);
            float Wv = fmaf(fabsf(sm), 9.5367431640625e-07f, sm);
            if (OPK) Wv = Wv / (m.sr * m.st);
            return Wv;
        };
        uint2 w = entry_or_end(a, item_at(0, a.lrun));
        uint2 wn = entry_or_end(a, item_at(1, a.lrun));
        Margins mc = load_margins(w);
        float W0 = width(mc, 0), W1 = width(mc, 1);
        auto is_active = [&](uint2 e) { return e.x != 0xffffffffu && ((e_mask(e) >> h) & 1u); };
        // Per block: wait for the accumulator, load and classify the two
        // 32-column chunks (one at a time, 32 live values), release the
        // accumulator, then count and stage band records before waiting for
        // the next block.  A tensor-memory load takes a few tens of cycles,
        // so nothing is gained by loading ahead; counting first keeps the
        // counting of one block from waiting on the next block's MMAs
        // (measured: that wait, placed before the counting, held the
        // epilogue a block behind the MMAs).
        uint32_t v[32];
        float mx = 0.0f;
        const uint32_t tq = tmem + ((q * 32u) << 16) + cg * 64u;
        for (uint64_t idx = 0; item_at(idx, a.lrun) < a.nwork; ++idx, ++it) {
            const uint32_t b = it & 1u, use = it >> 1;
            const uint2 wnn = entry_or_end(a, item_at(idx + 2, a.lrun));
            const Margins mn = load_margins(wn);
            const uint32_t I = e_row(w), J = e_col(w, h);
            const bool active = is_active(w);
            const bool diag = a.cross || (I == J);  // credit rows only
            const uint32_t taddr = tq + b * ACC_COLS;
            uint32_t in0 = 0, bd0 = 0, in1 = 0, bd1 = 0;
            bool busy0 = false, busy1 = false;
            if (!ptx::mbar_wait(&S.tfull[b], use & 1u, a.st, 30)) break;
            ptx::tc_fence_after();
            if (active) {
                ptx::tmem_ld_max_32x32b_x32(taddr, v, mx);
                ptx::tmem_ld_wait_regs(v, mx);
                busy0 = classify(v, mx, W0, in0, bd0);
                ptx::tmem_ld_max_32x32b_x32(taddr + 32u, v, mx);
                ptx::tmem_ld_wait_regs(v, mx);
            }
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&S.tempty[b]);
            if (active) busy1 = classify(v, mx, W1, in1, bd1);
            // the counts of buffer b were flushed and cleared for block it - 2
            if (!ptx::mbar_wait(&S.fdone[b], (use & 1u) ^ 1u, a.st, 32)) break;
            if (busy0 || busy1) {
                int* racc = S.rowacc[b];
                int* cacc = S.colacc[b];
                const uint32_t row = I * 128u + q * 32u + lane;
                const uint32_t col0 = J * 128u + (cg & 1u) * 64u;
                if (__any_sync(FULL, (bd0 | bd1) != 0)) stage_band(a, S, b, bd0, bd1, row, col0, diag, lane);
                if (!diag) {
                    col_counts(in0, cacc + cg * 64u, lane);
                    col_counts(in1, cacc + cg * 64u + 32u, lane);
                }
                const int rowcnt = __popc(in0) + __popc(in1);
                if (rowcnt) atomicAdd(&racc[q * 32u + lane], rowcnt);
                // the flusher skips the count arrays of blocks without in-pairs
                // (every lane takes part in the vote)
                const bool any_in = __any_sync(FULL, rowcnt != 0);
                if (lane == 0 && any_in) S.has_counts[b] = 1u;
                if (a.em.cnt) emit_in(a, in0, in1, row, col0, diag, lane);
            }
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&S.ebar[b]);
            W0 = width(mn, 0);
            W1 = width(mn, 1);
            w = wn;
            wn = wnn;
        }
    } else {
        // ------------------------------------------------ count flusher
        // adds the per-block row / column counts to global memory and clears
        // them, off the epilogue warps' critical path.  Band records go to
        // queue space the CTA reserves kResChunk records at a time: one
        // returning global atomic per chunk instead of one per block (its
        // round trip on every block made this warp the kernel's limit); the
        // unused tail of the last chunk is filled with empty records (mask 0,
        // no pairs), and band_records counts the real ones.
        constexpr uint32_t kResChunk = 4096;
        static_assert(kResChunk >= BAND_SMEM, "a block's records fit one new chunk");
        unsigned long long rbase = 0;
        uint32_t rleft = 0;
        // pairs (per lane) and records of the staged band records, added to
        // the status once at the end (two contended global atomics per block
        // otherwise)
        unsigned long long np_acc = 0, nrec_acc = 0;
        uint32_t it = 0;
        uint2 wnext = entry_or_end(a, item_at(0, a.lrun));
        for (uint64_t idx = 0;; ++idx, ++it) {
            if (item_at(idx, a.lrun) >= a.nwork) break;
            const uint32_t b = it & 1u, use = it >> 1;
            const uint2 w = wnext;
            wnext = entry_or_end(a, item_at(idx + 1, a.lrun));
            if (!ptx::mbar_wait(&S.ebar[b], use & 1u, a.st, 40)) break;
            int* racc = S.rowacc[b];
            int* cacc = S.colacc[b];
            const uint32_t col_a = e_col(w, 0) * 128u, col_b = e_col(w, 1) * 128u;
            // counts: only blocks with in-pairs wrote any (a column count
            // implies a row count), and only nonzero entries are cleared
            if (S.has_counts[b]) {
                int rv[4], cv[8];
#pragma unroll
                for (int e = 0; e < 4; ++e) rv[e] = racc[lane + 32 * e];
#pragma unroll
                for (int e = 0; e < 8; ++e) cv[e] = cacc[lane + 32 * e];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const uint32_t r = lane + 32 * e;
                    if (rv[e]) {
                        atomicAdd(&a.counts[e_row(w) * 128u + r], rv[e]);
                        racc[r] = 0;
                    }
                }
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const uint32_t c = lane + 32 * e;
                    if (cv[e]) {
                        atomicAdd(&a.counts[(c < 128u ? col_a : col_b - 128u) + c], cv[e]);
                        cacc[c] = 0;
                    }
                }
                __syncwarp();
                if (lane == 0) S.has_counts[b] = 0u;
            }
            // staged band records of this block: one global reservation, coalesced
            // copy, and their pair count
            const uint32_t nst = min(S.band_n[b], BAND_SMEM);
            if (nst) {
                // the first rleft records fill the current chunk, the rest
                // start a new one
                const bool grow = rleft < nst;
                unsigned long long nbase = 0;
                if (grow) {
                    if (lane == 0) nbase = atomicAdd(&a.st->band_count, (unsigned long long)kResChunk);
                    nbase = __shfl_sync(FULL, nbase, 0);
                }
                for (uint32_t e = lane; e < nst; e += 32) {
                    const BandRec r = S.band_buf[b][e];
                    np_acc += __popc(r.mask);
                    const unsigned long long g = e < rleft ? rbase + e : nbase + (e - rleft);
                    if (g < a.band_cap) a.band[g] = r;
                }
                nrec_acc += nst;
                if (grow) {
                    rbase = nbase + (nst - rleft);
                    rleft = kResChunk - (nst - rleft);
                } else {
                    rbase += nst;
                    rleft -= nst;
                }
            }
            __syncwarp();
            if (lane == 0) S.band_n[b] = 0;
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&S.fdone[b]);
        }
        // empty records in the unused tail of the last reserved chunk
        for (uint32_t e = lane; e < rleft; e += 32)
            if (rbase + e < a.band_cap) a.band[rbase + e] = BandRec{0u, 0u, 0u, 0u};
#pragma unroll
        for (int o = 16; o; o >>= 1) np_acc += __shfl_xor_sync(FULL, np_acc, o);
        if (lane == 0 && nrec_acc) {
            atomicAdd(&a.st->band_pairs, np_acc);
            atomicAdd(&a.st->band_records, nrec_acc);
        }
    }

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, TMEM_COLS);
    }
}

}  // namespace

int launch_gram16(const GramSide& A, const GramSide& B, const ScreenParams& P, const uint2* work,
                  uint64_t nwork, const float* cmax, const float* beta, const float* tsig,
                  const float* sig, bool cross, int32_t* counts, BandRec* band, uint64_t band_cap,
                  DevStatus* st, const Emit* em, int num_sms, cudaStream_t s) {
    if (nwork == 0) return EJOIN_OK;
    const bool fp8 = P.fmt == Fmt::E4M3;
    if (A.n_pad % 128 || B.n_pad % 256 || P.dp % (fp8 ? 128 : 64))
        return set_error(EJOIN_EINTERNAL, "gram: bad padding");
    if (A.n_pad > 0x7fffff00ull || B.n_pad > 0x7fffff00ull)
        return set_error(EJOIN_EUNSUPPORTED, "gram16: too many rows");
    CUtensorMap ma, mb, maa, mab;
    const CUtensorMapDataType adt =
        P.fmt == Fmt::FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    if (fp8) {
        EJ_TRY(make_tmap_2d(&ma, A.Q, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, P.width, A.n_pad, 128, 128));
        EJ_TRY(make_tmap_2d(&mb, B.Q, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, P.width, B.n_pad, 128, 128));
    } else {
        EJ_TRY(make_tmap_2d(&ma, A.Q, adt, 2, P.width, A.n_pad, 64, 128));
        EJ_TRY(make_tmap_2d(&mb, B.Q, adt, 2, P.width, B.n_pad, 64, 128));
    }
    EJ_TRY(make_tmap_2d(&maa, A.aug, adt, 2, 32, A.n_pad, 16, 128));
    EJ_TRY(make_tmap_2d(&mab, B.aug, adt, 2, 32, B.n_pad, 16, 128));
    GramArgs a;
    a.work = work;
    a.nwork = nwork;
    a.cmax = cmax;
    a.beta = beta;
    a.tsig = fp8 ? tsig : nullptr;
    a.sig = fp8 ? sig : nullptr;
    a.em = em ? *em : Emit{nullptr, 0, nullptr, 0, nullptr};
    a.cross = cross ? 1u : 0u;
    if (!cmax || !beta || (fp8 && (!tsig || !sig))) return set_error(EJOIN_EINTERNAL, "gram: margins missing");
    a.counts = counts;
    a.band = band;
    a.band_cap = band_cap;
    a.st = st;
    a.nhi = P.dp / (fp8 ? 128 : 64);
    a.split = P.split ? 1u : 0u;
    a.fmt = P.fmt == Fmt::BF16 ? 1u : 0u;
    // runs of consecutive entries per CTA (up to 16) while every CTA still gets
    // several runs
    uint32_t lrun = 4;
    while (lrun > 0 && nwork < (uint64_t)num_sms * (4ull << lrun)) --lrun;
    a.lrun = lrun;
    auto kern = fp8 ? gram_kernel<1> : gram_kernel<0>;
    EJ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    const uint64_t runs = (nwork + (1ull << lrun) - 1) >> lrun;
    const uint64_t grid = runs < (uint64_t)num_sms ? runs : (uint64_t)num_sms;
    kern<<<(unsigned)grid, NTHREADS, SMEM_BYTES, s>>>(ma, mb, maa, mab, a);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

}  // namespace ejoin
