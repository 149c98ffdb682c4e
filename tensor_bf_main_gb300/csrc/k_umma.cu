// k_umma.cu -- the tcgen05 Gram screen (EJOIN_BF16 / BF16_SPLIT / FP16).
//
// Re-designs the reference's main tensor path,
// distanceCalculationBruteForceTensorHalf (kernel_join.cu:328-524): there a
// warp computes -2*Q*C^T + |c|^2 for 16 queries x 16 candidates per wmma
// m16n16k16, round-trips every k-chunk through shared memory, re-adds the
// query norms in scalar code and bumps one global counter per hit with
// sqrt(|d2|) <= eps.  Here:
//
//  * A persistent CTA per SM walks a list of 128x128 tile pairs (I <= J, the
//    upper triangle only).  Warp 0 streams K-slabs of both row blocks into a
//    6-stage shared-memory ring with TMA (128-byte swizzle).  One thread of
//    warp 1 issues tcgen05.mma (M=128, N=128, K=16 per instruction) into one
//    of two FP32 accumulators in tensor memory, so the next tile's MMAs run
//    while 8 epilogue warps read the previous one.
//  * Operand rows are [hi | lo | aug] (k_prep.cu).  With the hi+lo split the
//    MMAs form hi*hi + hi*lo + lo*hi.  The aug slab adds -alpha_i - alpha_j,
//    so the accumulator holds C_ij = q_i.q_j - alpha_i - alpha_j and the
//    rigorous screen is a sign test:
//        C >= 0          pair certainly within eps        (counted)
//        C < -W_IJ       pair certainly outside eps
//        otherwise       band: queued for the FP64 recheck
//    W_IJ = max beta over tile I + max beta over tile J.
//  * The epilogue packs sign bits with one funnel shift per element, counts
//    rows with popc, transposes the 32x32 bit block across the warp to count
//    columns (off-diagonal tiles credit both points), and flushes per-point
//    counts once per tile.  No distance ever reaches global memory.
//
// Every wait is bounded (umma_ptx.cuh); on expiry all roles stop, in-flight
// copies and MMAs are drained (bounded) and tensor memory is freed.
#include "tmap.cuh"
#include "umma_ptx.cuh"

namespace ejoin {
namespace {

constexpr int NST = 5;                      // smem ring stages
constexpr int SLAB_BYTES = 128 * 128;       // 128 rows x 128 bytes
constexpr int AUG_BYTES = 128 * 32;         // 128 rows x 32 bytes (16 elements)
// A slab | B slab | A aug | B aug; the aug boxes are loaded with the first
// slab of every tile only
constexpr int STAGE_BYTES = 2 * SLAB_BYTES + 2 * AUG_BYTES;
constexpr uint32_t DATA_TX = 2 * SLAB_BYTES;
constexpr uint32_t FIRST_TX = 2 * SLAB_BYTES + 2 * AUG_BYTES;
constexpr int NUM_EPI_WARPS = 16;          // 4 per SM sub-partition (latency hiding)
constexpr int FLUSH_WARP = 2 + NUM_EPI_WARPS;  // adds the per-tile counts to global memory
constexpr int NTHREADS = (3 + NUM_EPI_WARPS) * 32;
constexpr uint32_t TMEM_COLS = 256;         // two 128x128 FP32 accumulators
constexpr uint32_t FULL = 0xffffffffu;

struct GramArgs {
    const uint2* work;
    uint64_t nwork;
    const float* tmax;
    const float* tsig;  // FP8: per-tile minimum row scale (null for 16-bit operands)
    int32_t* counts;
    BandPair* band;
    uint64_t band_cap;
    DevStatus* st;
    uint32_t nhi;    // 64-element data slabs per part
    uint32_t split;  // hi + lo
    uint32_t fmt;    // 16-bit operands: 0 = FP16, 1 = BF16 (instruction-descriptor format)
};

// Band width of tile pair (I, J): beta_i + beta_j <= W (Gram units; FP8
// operands: divided by sigma_I sigma_J, the accumulator's unit).  The sum is
// rounded up by the 2^-20 relative margin; division by the power-of-two
// scales is exact.
__device__ __forceinline__ float band_width(const GramArgs& a, uint2 w) {
    const float s = __ldg(&a.tmax[w.x]) + __ldg(&a.tmax[w.y]);
    float W = fmaf(fabsf(s), 9.5367431640625e-07f, s);
    if (a.tsig) W = W / (__ldg(&a.tsig[w.x]) * __ldg(&a.tsig[w.y]));
    return W;
}

constexpr uint32_t BAND_SMEM = 1024;  // staged band entries per accumulator buffer
constexpr uint32_t BAND_SKIP = 0xffffffffu;  // staged slot not used (recheck skips i >= n)

struct Ctl {
    uint64_t full[NST], empty[NST];
    uint64_t tfull[2], tempty[2];
    uint64_t ebar[2];   // epilogue warps done with the counts of buffer b
    uint64_t fdone[2];  // flusher done with (and cleared) the counts of buffer b
    uint64_t fin;
    uint32_t tmem_base;
    int rowacc[2][128];
    int colacc[2][128];
    uint32_t band_n[2];                  // band entries staged for buffer b
    BandPair band_buf[2][BAND_SMEM];     // staged band entries (flushed by the flusher warp)
};

constexpr size_t SMEM_BYTES = 1024 + (size_t)NST * STAGE_BYTES + sizeof(Ctl);

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

// Element offset of K-slab `step` of a tile: [hi0, lo0, hi1, lo1, ...] with the
// split, [hi0, hi1, ...] without.
template <int OPK>
__device__ __forceinline__ uint32_t slab_x(uint32_t step, uint32_t nhi, uint32_t split) {
    constexpr uint32_t E = OPK ? 128u : 64u;  // elements per 128-byte slab row
    if (split) return (step & 1) ? E * nhi + E * (step >> 1) : E * (step >> 1);
    return E * step;
}

// OPK 0: 16-bit operands, data MMAs kind::f16; OPK 1: E4M3 operands, data
// MMAs kind::f8f6f4 (K = 32 per instruction, same 32-byte k-steps), the aug
// MMA stays kind::f16 in BF16 and accumulates into the same tensor memory.
template <int OPK>
__global__ void __launch_bounds__(NTHREADS, 1)
    gram_kernel(const __grid_constant__ CUtensorMap tq, const __grid_constant__ CUtensorMap taug,
                const GramArgs a) {
    extern __shared__ uint8_t smraw[];
    uint8_t* stages = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
    Ctl& S = *reinterpret_cast<Ctl*>(stages + (size_t)NST * STAGE_BYTES);
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
        for (int b = 0; b < 2; ++b) {
            ptx::mbar_init(&S.tfull[b], 1);
            ptx::mbar_init(&S.tempty[b], NUM_EPI_WARPS);
            ptx::mbar_init(&S.ebar[b], NUM_EPI_WARPS);
            ptx::mbar_init(&S.fdone[b], 1);
        }
        ptx::mbar_init(&S.fin, 1);
        ptx::fence_barrier_init();
        ptx::tma_prefetch_desc(&tq);
        ptx::tma_prefetch_desc(&taug);
    }
    for (int i = threadIdx.x; i < 512; i += NTHREADS) (&S.rowacc[0][0])[i] = 0;
    if (threadIdx.x < 2) S.band_n[threadIdx.x] = 0;
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
            bool ok = true;
            uint2 wn = blockIdx.x < a.nwork ? __ldg(&a.work[blockIdx.x]) : make_uint2(0, 0);
            for (uint64_t u = blockIdx.x; u < a.nwork && ok; u += gridDim.x) {
                const uint2 w = wn;
                if (u + gridDim.x < a.nwork) wn = __ldg(&a.work[u + gridDim.x]);  // prefetch
                for (uint32_t step = 0; step < nsteps; ++step) {
                    if (!ptx::mbar_wait(&S.empty[st], ph ^ 1u, a.st, 10)) {
                        ok = false;
                        break;
                    }
                    uint8_t* sa = stages + (size_t)st * STAGE_BYTES;
                    const int32_t x = (int32_t)slab_x<OPK>(step, a.nhi, a.split);
                    ptx::mbar_arrive_expect_tx(&S.full[st], step == 0 ? FIRST_TX : DATA_TX);
                    ptx::tma_load_2d(sa, &tq, x, (int32_t)(w.x * 128u), &S.full[st]);
                    ptx::tma_load_2d(sa + SLAB_BYTES, &tq, x, (int32_t)(w.y * 128u), &S.full[st]);
                    if (step == 0) {
                        ptx::tma_load_2d(sa + 2 * SLAB_BYTES, &taug, 0, (int32_t)(w.x * 128u),
                                         &S.full[st]);
                        ptx::tma_load_2d(sa + 2 * SLAB_BYTES + AUG_BYTES, &taug, 16,
                                         (int32_t)(w.y * 128u), &S.full[st]);
                    }
                    issued_ph[st] = ph;
                    ++issued;
                    if (++st == NST) {
                        st = 0;
                        ph ^= 1u;
                    }
                }
            }
            // drain: every issued copy has landed before the CTA can exit
            const uint32_t last = issued < NST ? issued : NST;
            for (uint32_t k = 0; k < last; ++k) {
                const uint32_t s = (st + NST - 1 - k) % NST;
                ptx::mbar_wait(&S.full[s], issued_ph[s], a.st, 11);
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t idesc =
                OPK ? ptx::idesc_f32acc(0, 0, 128, 128) : ptx::idesc_f32acc(a.fmt, a.fmt, 128, 128);
            const uint32_t idesc_aug =
                OPK ? ptx::idesc_f32acc(1, 1, 128, 128) : idesc;
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
            for (uint64_t u = blockIdx.x; u < a.nwork && ok; u += gridDim.x, ++it) {
                const uint32_t b = it & 1u, use = it >> 1;
                if (!ptx::mbar_wait(&S.tempty[b], (use & 1u) ^ 1u, a.st, 21)) break;
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem + b * 128u;
                uint32_t acc = 0;
                for (uint32_t c = 0; c < a.nhi && ok; ++c) {
                    uint32_t s_hi, s_lo = 0;
                    if (!take(s_hi)) { ok = false; break; }
                    if (a.split && !take(s_lo)) { ok = false; break; }
                    ptx::tc_fence_after();
                    uint8_t* st_hi = stages + (size_t)s_hi * STAGE_BYTES;
                    const uint64_t ah = ptx::sdesc_sw128(ptx::smem_u32(st_hi));
                    const uint64_t bh = ptx::sdesc_sw128(ptx::smem_u32(st_hi + SLAB_BYTES));
                    if (c == 0) {
                        // aug: A side (alpha_i, -1) x B side (-1, alpha_j), one K = 16 step
                        const uint64_t aa = ptx::sdesc_sw32(ptx::smem_u32(st_hi + 2 * SLAB_BYTES));
                        const uint64_t ba =
                            ptx::sdesc_sw32(ptx::smem_u32(st_hi + 2 * SLAB_BYTES + AUG_BYTES));
                        ptx::mma_f16(d_tmem, aa, ba, idesc_aug, 0);
                        acc = 1;
                    }
                    if (a.split) {
                        uint8_t* st_lo = stages + (size_t)s_lo * STAGE_BYTES;
                        const uint64_t al = ptx::sdesc_sw128(ptx::smem_u32(st_lo));
                        const uint64_t bl = ptx::sdesc_sw128(ptx::smem_u32(st_lo + SLAB_BYTES));
#pragma unroll
                        for (uint32_t kk = 0; kk < 4; ++kk) {
                            mma(d_tmem, ah + 2 * kk, bh + 2 * kk, acc);
                            mma(d_tmem, ah + 2 * kk, bl + 2 * kk, 1);
                            mma(d_tmem, al + 2 * kk, bh + 2 * kk, 1);
                        }
                        ptx::mma_commit(&S.empty[s_hi]);
                        ptx::mma_commit(&S.empty[s_lo]);
                    } else {
#pragma unroll
                        for (uint32_t kk = 0; kk < 4; ++kk) mma(d_tmem, ah + 2 * kk, bh + 2 * kk, acc);
                        ptx::mma_commit(&S.empty[s_hi]);
                    }
                }
                if (!ok) break;
                ptx::mma_commit(&S.tfull[b]);
            }
            // drain: all MMAs complete before tensor memory is freed
            ptx::mma_commit(&S.fin);
            ptx::mbar_wait(&S.fin, 0, a.st, 22);
        }
    } else if (warp < FLUSH_WARP) {
        // ------------------------------------------------ epilogue warps
        // warp e reads lane quarter (warp % 4) and the 32 columns 32 * (e / 4)
        const uint32_t ew = warp - 2;          // 0..15
        const uint32_t q = warp & 3u;          // tensor-memory lane quarter
        const uint32_t cg = ew >> 2;           // column group
        uint32_t it = 0;
        // the next tile's (I, J) and margins are loaded one tile ahead, so
        // their latency hides behind the current tile
        uint2 w = blockIdx.x < a.nwork ? __ldg(&a.work[blockIdx.x]) : make_uint2(0, 0);
        float W = blockIdx.x < a.nwork ? band_width(a, w) : 0.0f;
        for (uint64_t u = blockIdx.x; u < a.nwork; u += gridDim.x, ++it) {
            const uint32_t b = it & 1u, use = it >> 1;
            const bool has_next = u + gridDim.x < a.nwork;
            uint2 wn = make_uint2(0, 0);
            if (has_next) wn = __ldg(&a.work[u + gridDim.x]);
            const bool diag = (w.x == w.y);
            if (!ptx::mbar_wait(&S.tfull[b], use & 1u, a.st, 30)) break;
            ptx::tc_fence_after();
            uint32_t v[32];
            ptx::tmem_ld_32x32b_x32(tmem + ((q * 32u) << 16) + b * 128u + cg * 32u, v);
            const float Wn = has_next ? band_width(a, wn) : 0.0f;
            ptx::tmem_ld_wait();
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&S.tempty[b]);

            // Fast path: if max + W < 0 for the whole 32 x 32 chunk, every
            // pair in it is certainly out (rounding of the FP32 add is
            // monotone, so max + W >= 0 whenever any element is >= -W).
            float m8[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
                m8[j] = fmaxf(fmaxf(__uint_as_float(v[j]), __uint_as_float(v[j + 8])),
                              fmaxf(__uint_as_float(v[j + 16]), __uint_as_float(v[j + 24])));
            const float mx = fmaxf(fmaxf(fmaxf(m8[0], m8[1]), fmaxf(m8[2], m8[3])),
                                   fmaxf(fmaxf(m8[4], m8[5]), fmaxf(m8[6], m8[7])));
            const bool busy = __any_sync(FULL, mx + W >= 0.0f);
            uint32_t inm = 0, bandm = 0;
            if (busy) {
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
            }
            // the counts of buffer b were flushed and cleared for tile it - 2
            if (!ptx::mbar_wait(&S.fdone[b], (use & 1u) ^ 1u, a.st, 32)) break;
            if (busy) {
                int* racc = S.rowacc[b];
                int* cacc = S.colacc[b];
                const uint32_t row = w.x * 128u + q * 32u + lane;
                const uint32_t col0 = w.y * 128u + cg * 32u;
                if (__any_sync(FULL, bandm != 0)) {
                    // stage in shared memory (the flusher reserves global slots)
                    const uint32_t nb = __popc(bandm);
                    uint32_t incl = nb;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t t = __shfl_up_sync(FULL, incl, o);
                        if (lane >= (uint32_t)o) incl += t;
                    }
                    const uint32_t total = __shfl_sync(FULL, incl, 31);
                    uint32_t base = 0;
                    if (lane == 31) base = atomicAdd(&S.band_n[b], total);
                    base = __shfl_sync(FULL, base, 31);
                    const bool fits = base + total <= BAND_SMEM;  // warp-uniform
                    uint32_t slot = base + incl - nb;
                    unsigned long long gslot = fits ? 0ull : band_reserve(a.st, nb);
                    uint32_t m = bandm;
                    while (m) {
                        const uint32_t c = __ffs(m) - 1;
                        m &= m - 1;
                        BandPair bp;
                        bp.i = row;
                        bp.j = (col0 + c) | (diag ? 0u : kBandBoth);
                        if (fits) {
                            S.band_buf[b][slot++] = bp;
                        } else {
                            if (gslot < a.band_cap) a.band[gslot] = bp;
                            ++gslot;
                        }
                    }
                    if (!fits) {
                        // mark this warp's staged slots unused
                        for (uint32_t q2 = base + incl - nb; q2 < base + incl && q2 < BAND_SMEM; ++q2)
                            S.band_buf[b][q2] = BandPair{BAND_SKIP, BAND_SKIP};
                    }
                }
                if (__any_sync(FULL, inm != 0)) {
                    if (!diag) {
                        const int cc = __popc(transpose32(inm, lane));
                        if (cc) atomicAdd(&cacc[cg * 32u + lane], cc);
                    }
                    const int rowcnt = __popc(inm);
                    if (rowcnt) atomicAdd(&racc[q * 32u + lane], rowcnt);
                }
            }
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&S.ebar[b]);
            W = Wn;
            w = wn;
        }
    } else {
        // ------------------------------------------------ count flusher
        // adds the per-tile row / column counts to global memory and clears
        // them, off the epilogue warps' critical path
        uint32_t it = 0;
        for (uint64_t u = blockIdx.x; u < a.nwork; u += gridDim.x, ++it) {
            const uint32_t b = it & 1u, use = it >> 1;
            const uint2 w = __ldg(&a.work[u]);
            if (!ptx::mbar_wait(&S.ebar[b], use & 1u, a.st, 40)) break;
            int* racc = S.rowacc[b];
            int* cacc = S.colacc[b];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const uint32_t r = lane + 32 * e;
                const int rv = racc[r];
                if (rv) atomicAdd(&a.counts[w.x * 128u + r], rv);
                racc[r] = 0;
                const int cv = cacc[r];
                if (cv) atomicAdd(&a.counts[w.y * 128u + r], cv);
                cacc[r] = 0;
            }
            // staged band entries of this tile: one global reservation, coalesced copy
            const uint32_t nst = min(S.band_n[b], BAND_SMEM);
            if (nst) {
                unsigned long long gbase = 0;
                if (lane == 0) gbase = atomicAdd(&a.st->band_count, (unsigned long long)nst);
                gbase = __shfl_sync(FULL, gbase, 0);
                for (uint32_t e = lane; e < nst; e += 32)
                    if (gbase + e < a.band_cap) a.band[gbase + e] = S.band_buf[b][e];
            }
            __syncwarp();
            if (lane == 0) S.band_n[b] = 0;
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&S.fdone[b]);
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

int launch_gram16(const void* Q, const void* aug, uint64_t n_pad, const ScreenParams& P,
                  const uint2* work, uint64_t nwork, const float* tmax, const float* tsig,
                  int32_t* counts, BandPair* band, uint64_t band_cap, DevStatus* st, int num_sms,
                  cudaStream_t s) {
    if (nwork == 0) return EJOIN_OK;
    const bool fp8 = P.fmt == Fmt::E4M3;
    if (n_pad % 128 || P.dp % (fp8 ? 128 : 64)) return set_error(EJOIN_EINTERNAL, "gram: bad padding");
    if (n_pad > 0x7fffff80ull) return set_error(EJOIN_EUNSUPPORTED, "gram16: too many rows");
    CUtensorMap map, amap;
    const CUtensorMapDataType adt =
        P.fmt == Fmt::FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    if (fp8)
        EJ_TRY(make_tmap_2d(&map, Q, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, P.width, n_pad, 128, 128));
    else
        EJ_TRY(make_tmap_2d(&map, Q, adt, 2, P.width, n_pad, 64, 128));
    EJ_TRY(make_tmap_2d(&amap, aug, adt, 2, 32, n_pad, 16, 128));
    GramArgs a;
    a.work = work;
    a.nwork = nwork;
    a.tmax = tmax;
    a.tsig = fp8 ? tsig : nullptr;
    a.counts = counts;
    a.band = band;
    a.band_cap = band_cap;
    a.st = st;
    a.nhi = P.dp / (fp8 ? 128 : 64);
    a.split = P.split ? 1u : 0u;
    a.fmt = P.fmt == Fmt::BF16 ? 1u : 0u;
    auto kern = fp8 ? gram_kernel<1> : gram_kernel<0>;
    EJ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    const uint64_t grid = nwork < (uint64_t)num_sms ? nwork : (uint64_t)num_sms;
    kern<<<(unsigned)grid, NTHREADS, SMEM_BYTES, s>>>(map, amap, a);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

}  // namespace ejoin
