// k_direct.cu -- FP64 CUDA-core kernels with the reference's exact arithmetic.
//
//  * direct_selfjoin_kernel: the exact arbiter (EJOIN_FP64_DIRECT, reference
//    searchMode 1, kernel_join.cu:168-200).  The reference runs one thread
//    per query over all N candidates and bumps one global 64-bit counter per
//    hit; here a CTA takes one 64x64 tile pair of the upper triangle (I <= J),
//    stages both row blocks in shared memory k-chunk by k-chunk, every thread
//    keeps a 4x4 block of independent FP64 chains, and the hits become
//    per-point counts (row counts for I, column counts for J when I < J).
//    d2(a, b) and d2(b, a) are bitwise equal ((a-b)^2 == (b-a)^2), so the
//    upper triangle is exact.
//  * direct_query_kernel: the same tile over (query rows) x (all points).
//  * band_recheck_kernel: one thread per band pair, the same chain.
//
// Every chain follows the reference's compiled arithmetic (exact_d2:
// fma(t0, t0, fl(t1*t1)), then fma(t, t, acc) in index order).  Zero padding
// of the k loop is exact: fma(0, 0, acc) == acc for acc >= +0.
#include <cuda_fp16.h>

#include <algorithm>

#include "ejoin_internal.cuh"

namespace ejoin {
namespace {

constexpr int TB = 64;        // tile edge (points)
constexpr int KC = 32;        // k-chunk staged per step
constexpr int PADK = TB + 1;  // smem row pitch (doubles) of the k-major stage

// Stage rows [r0, r0+64) x coords [k0, k0+KC) of X (row stride ld) into
// S[k][r] (k-major).  rows >= n and coords >= d are zero.
__device__ __forceinline__ void stage_tile(double (*S)[PADK], const double* __restrict__ X,
                                           uint64_t n, uint32_t d, uint64_t r0, uint32_t k0,
                                           const uint64_t* __restrict__ rowmap, uint64_t nmap) {
    for (int e = threadIdx.x; e < TB * KC; e += blockDim.x) {
        int r = e / KC, k = e % KC;
        uint64_t row = r0 + r;
        uint32_t kk = k0 + k;
        double v = 0.0;
        if (rowmap) {
            if (row < nmap && kk < d) v = X[rowmap[row] * (uint64_t)d + kk];
        } else if (row < n && kk < d) {
            v = X[row * (uint64_t)d + kk];
        }
        S[k][r] = v;
    }
}

// One 64x64 tile of exact squared distances.  Thread (ty, tx) owns rows
// ty + 16*rr and columns tx + 16*cc.  The first chunk (first) starts every
// chain with fma(t0, t0, fl(t1*t1)), the reference's compiled form of its
// first two terms (exact_d2); zero-padded coordinates give t = 0 there too.
__device__ __forceinline__ void tile_chains(double acc[4][4], double (*SA)[PADK],
                                            double (*SB)[PADK], int ty, int tx, bool first) {
    int k0 = 0;
    if (first) {
        double a0[4], a1[4], b0[4], b1[4];
#pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
            a0[rr] = SA[0][ty + 16 * rr];
            a1[rr] = SA[1][ty + 16 * rr];
        }
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
            b0[cc] = SB[0][tx + 16 * cc];
            b1[cc] = SB[1][tx + 16 * cc];
        }
#pragma unroll
        for (int rr = 0; rr < 4; ++rr)
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
                const double t0 = __dsub_rn(a0[rr], b0[cc]);
                const double t1 = __dsub_rn(a1[rr], b1[cc]);
                acc[rr][cc] = __fma_rn(t0, t0, __dmul_rn(t1, t1));
            }
        k0 = 2;
    }
#pragma unroll 4
    for (int k = k0; k < KC; ++k) {
        double a[4], b[4];
#pragma unroll
        for (int rr = 0; rr < 4; ++rr) a[rr] = SA[k][ty + 16 * rr];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) b[cc] = SB[k][tx + 16 * cc];
#pragma unroll
        for (int rr = 0; rr < 4; ++rr)
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
                double t = __dsub_rn(a[rr], b[cc]);
                acc[rr][cc] = __fma_rn(t, t, acc[rr][cc]);
            }
    }
}

__global__ void __launch_bounds__(256) direct_selfjoin_kernel(const double* __restrict__ X,
                                                              uint64_t n, uint32_t d, double T,
                                                              uint64_t nT, uint64_t tiles,
                                                              int32_t* counts, Emit em) {
    __shared__ double SA[KC][PADK];
    __shared__ double SB[KC][PADK];
    __shared__ int rowc[TB], colc[TB];
    const uint64_t t = blockIdx.x + (uint64_t)blockIdx.y * gridDim.x;
    if (t >= tiles) return;
    uint64_t I, J;
    tri_decode(t, nT, I, J);
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    if (threadIdx.x < TB) {
        rowc[threadIdx.x] = 0;
        colc[threadIdx.x] = 0;
    }
    double acc[4][4];
#pragma unroll
    for (int rr = 0; rr < 4; ++rr)
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) acc[rr][cc] = 0.0;
    for (uint32_t k0 = 0; k0 < d; k0 += KC) {
        __syncthreads();
        stage_tile(SA, X, n, d, I * TB, k0, nullptr, 0);
        stage_tile(SB, X, n, d, J * TB, k0, nullptr, 0);
        __syncthreads();
        tile_chains(acc, SA, SB, ty, tx, k0 == 0);
    }
    const bool diag = (I == J);
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
        uint64_t i = I * TB + ty + 16 * rr;
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
            uint64_t j = J * TB + tx + 16 * cc;
            if (i < n && j < n && acc[rr][cc] <= T) {
                atomicAdd(&rowc[ty + 16 * rr], 1);
                if (!diag) atomicAdd(&colc[tx + 16 * cc], 1);
                emit_pair(em, BandPair{(uint32_t)i, (uint32_t)j | (diag ? 0u : kBandBoth)});
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < TB) {
        uint64_t i = I * TB + threadIdx.x, j = J * TB + threadIdx.x;
        if (rowc[threadIdx.x] && i < n) atomicAdd(&counts[i], rowc[threadIdx.x]);
        if (colc[threadIdx.x] && j < n) atomicAdd(&counts[j], colc[threadIdx.x]);
    }
}

// Query rows: rows[q] of X, or (Xq non-null) row q of a separate array Xq.
__global__ void __launch_bounds__(256) direct_query_kernel(const double* __restrict__ X, uint64_t n,
                                                           uint32_t d, double T,
                                                           const uint64_t* __restrict__ rows,
                                                           const double* __restrict__ Xq,
                                                           uint64_t nq, int32_t* counts) {
    __shared__ double SA[KC][PADK];
    __shared__ double SB[KC][PADK];
    __shared__ int rowc[TB];
    const uint64_t Q = blockIdx.y, J = blockIdx.x;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    if (threadIdx.x < TB) rowc[threadIdx.x] = 0;
    double acc[4][4];
#pragma unroll
    for (int rr = 0; rr < 4; ++rr)
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) acc[rr][cc] = 0.0;
    for (uint32_t k0 = 0; k0 < d; k0 += KC) {
        __syncthreads();
        if (Xq) stage_tile(SA, Xq, nq, d, Q * TB, k0, nullptr, 0);
        else stage_tile(SA, X, n, d, Q * TB, k0, rows, nq);
        stage_tile(SB, X, n, d, J * TB, k0, nullptr, 0);
        __syncthreads();
        tile_chains(acc, SA, SB, ty, tx, k0 == 0);
    }
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
        uint64_t q = Q * TB + ty + 16 * rr;
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
            uint64_t j = J * TB + tx + 16 * cc;
            if (q < nq && j < n && acc[rr][cc] <= T) atomicAdd(&rowc[ty + 16 * rr], 1);
        }
    }
    __syncthreads();
    if (threadIdx.x < TB) {
        uint64_t q = Q * TB + threadIdx.x;
        if (rowc[threadIdx.x] && q < nq) atomicAdd(&counts[q], rowc[threadIdx.x]);
    }
}

__global__ void __launch_bounds__(256) band_recheck_kernel(const double* __restrict__ X, uint32_t d,
                                                           const uint32_t* __restrict__ perm,
                                                           double T,
                                                           const BandPair* __restrict__ band,
                                                           uint64_t nband, uint64_t n,
                                                           int32_t* counts, DevStatus* st) {
    uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    unsigned hit = 0;
    BandPair bp = {0u, 0u};
    if (e < nband) bp = band[e];
    const uint32_t i = bp.i, j = bp.j & ~kBandBoth;
    // padding rows (index >= n) hold no point: such pairs are never neighbours
    if (e < nband && i < n && j < n) {
        uint64_t oi = perm ? perm[i] : i, oj = perm ? perm[j] : j;
        double d2 = exact_d2(X + oi * (uint64_t)d, X + oj * (uint64_t)d, d);
        if (d2 <= T) {
            hit = 1;
            atomicAdd(&counts[i], 1);
            if (bp.j & kBandBoth) atomicAdd(&counts[j], 1);
        }
    }
    unsigned c = __reduce_add_sync(0xffffffffu, hit);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&st->band_hits, (unsigned long long)c);
}

// Two-stage recheck of the band of the tensor-core screen.  For every band
// pair, S = sum_c fl32(zf_ic - zf_jc)^2 over the FP32 coordinates of the
// packed rows (any summation order: the bound covers it), then a rigorous
// decision that scales with the pair's own distance:
//   |w| = |zf_i - zf_j| differs from the exact scaled distance by at most
//   rad_i + rad_j, and S from |w|^2 by the relative c32 (+ abs32), so
//   S / (1 - c32) <= (sqrt(Tlo) - rad)^2   => neighbour
//   S / (1 + c32) >  (sqrt(Thi) + rad)^2   => not a neighbour
// i.e. S + abs32 <= (sqrt(Tlo) - rad)^2 (1 - c32) and
//      S - abs32 >  (sqrt(Thi) + rad)^2 (1 + c32).
// Both tests run in FP32 with every operation rounded in the safe direction
// (the constants are rounded outward on the host), so they stay rigorous
// without FP64, whose throughput on GB300 is a small fraction of FP32's.  An
// infinite radius (bad or padding row) decides nothing.
// Only the pairs left undecided (a tiny fraction) run the exact FP64 chain of
// the reference arithmetic on the original rows.  Returns whether (i, j) is a
// neighbour pair; counts the exact runs.
__device__ __forceinline__ bool recheck_decide(const double* __restrict__ X, uint32_t d,
                                               const uint32_t* __restrict__ perm, double T,
                                               const Recheck32& R, uint32_t i, uint32_t j,
                                               float S, unsigned& exact_runs) {
    const float rr = __fadd_ru(R.rad[i], R.radb[j]);
    const float lo = __fsub_rd(R.f_sTlo, rr);
    if (lo >= 0.0f && __fadd_ru(S, R.f_abs) <= __fmul_rd(__fmul_rd(lo, lo), R.f_kin)) return true;
    const float hi = __fadd_ru(R.f_sThi, rr);
    if (__fsub_rd(S, R.f_abs) > __fmul_ru(__fmul_ru(hi, hi), R.f_kout)) return false;
    ++exact_runs;
    const uint64_t oi = perm ? perm[i] : i, oj = R.permb ? R.permb[j] : j;
    return exact_d2(X + oi * (uint64_t)d, R.Xb + oj * (uint64_t)d, d) <= T;
}

__device__ __forceinline__ void recheck_totals(DevStatus* st, unsigned hits, unsigned exact_runs) {
    const unsigned c = __reduce_add_sync(0xffffffffu, hits);
    const unsigned x = __reduce_add_sync(0xffffffffu, exact_runs);
    if ((threadIdx.x & 31) == 0) {
        if (c) atomicAdd(&st->band_hits, (unsigned long long)c);
        if (x) atomicAdd(&st->exact_rechecks, (unsigned long long)x);
    }
}

// Read-only row loads that do not allocate in L1: the band rows are
// gathered with little reuse, and allocating them thrashed L1 (measured on
// c4: the recheck ran 1.4x faster without allocation).  32 bytes (p 32-byte
// aligned) or 16 bytes (p 16-byte aligned).
__device__ __forceinline__ void ldg8(const float* p, float (&r)[8]) {
    asm("ld.global.nc.L1::no_allocate.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]),
          "=f"(r[7])
        : "l"(p));
}
// cached forms, for the row a warp reuses across consecutive pairs
__device__ __forceinline__ void ldg8c(const float* p, float (&r)[8]) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]),
          "=f"(r[7])
        : "l"(p));
}
__device__ __forceinline__ float4 ldg4(const float* p) {
    float4 r;
    asm("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
        : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
        : "l"(p));
    return r;
}

// Short rows (d <= 64, 16-byte aligned): a thread per pair streams both rows
// with 16-byte loads, or 32-byte loads when V8 (four partial sums): 32 pairs
// in flight per warp.  The kernel is bound by L1 wavefronts (each lane reads
// its own row), so wider loads move more bytes per wavefront.
template <bool V8>
__global__ void __launch_bounds__(256) band_recheck_thread_kernel(const double* __restrict__ X,
                                                                  uint32_t d,
                                                                  const uint32_t* __restrict__ perm,
                                                                  double T, Recheck32 R,
                                                                  const BandPair* __restrict__ band,
                                                                  uint64_t nband, uint64_t n,
                                                                  int32_t* counts, DevStatus* st,
                                                                  Emit em) {
    unsigned hits = 0, exact_runs = 0;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nband;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const BandPair bp = band[e];
        const uint32_t i = bp.i, j = bp.j & ~kBandBoth;
        if (i >= n || j >= R.nb) continue;
        float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
        if (V8) {
            const float* a = R.Xf + (uint64_t)i * d;
            const float* b = R.Xfb + (uint64_t)j * d;
#pragma unroll 2
            for (uint32_t c = 0; c < d; c += 8) {
                float u[8], v[8];
                ldg8(a + c, u);
                ldg8(b + c, v);
#pragma unroll
                for (int k = 0; k < 8; k += 4) {
                    const float t0 = u[k] - v[k], t1 = u[k + 1] - v[k + 1];
                    const float t2 = u[k + 2] - v[k + 2], t3 = u[k + 3] - v[k + 3];
                    s0 = fmaf(t0, t0, s0);
                    s1 = fmaf(t1, t1, s1);
                    s2 = fmaf(t2, t2, s2);
                    s3 = fmaf(t3, t3, s3);
                }
            }
        } else {
            const float4* a = reinterpret_cast<const float4*>(R.Xf + (uint64_t)i * d);
            const float4* b = reinterpret_cast<const float4*>(R.Xfb + (uint64_t)j * d);
#pragma unroll 4
            for (uint32_t c = 0; c < d / 4; ++c) {
                const float4 u = ldg4(reinterpret_cast<const float*>(a + c));
                const float4 v = ldg4(reinterpret_cast<const float*>(b + c));
                const float t0 = u.x - v.x, t1 = u.y - v.y, t2 = u.z - v.z, t3 = u.w - v.w;
                s0 = fmaf(t0, t0, s0);
                s1 = fmaf(t1, t1, s1);
                s2 = fmaf(t2, t2, s2);
                s3 = fmaf(t3, t3, s3);
            }
        }
        if (recheck_decide(X, d, perm, T, R, i, j, (s0 + s1) + (s2 + s3), exact_runs)) {
            atomicAdd(&counts[i], 1);
            if (bp.j & kBandBoth) atomicAdd(&counts[j], 1);
            emit_pair(em, bp);
            ++hits;
        }
    }
    recheck_totals(st, hits, exact_runs);
}

// First decision of a band pair from the FP16 copies (S = their squared
// distance, computed in FP32 like the FP32 one: the conversions are exact):
// 1 = in, 0 = out, -1 = undecided.  The copies' radii (rad + |zh - zf|)
// replace the FP32 radii; otherwise the same directed-rounding tests as
// recheck_decide.
__device__ __forceinline__ int decide16(const Recheck32& R, uint32_t i, uint32_t j, float S) {
    const float rr = __fadd_ru(R.radh[i], R.radhb[j]);
    const float lo = __fsub_rd(R.f_sTlo, rr);
    if (lo >= 0.0f && __fadd_ru(S, R.f_abs) <= __fmul_rd(__fmul_rd(lo, lo), R.f_kin)) return 1;
    const float hi = __fadd_ru(R.f_sThi, rr);
    if (__fsub_rd(S, R.f_abs) > __fmul_ru(__fmul_ru(hi, hi), R.f_kout)) return 0;
    return -1;
}

// 8 FP16 values (16 bytes, p 16-byte aligned): the cached form for the row a
// warp reuses, the no-allocate form for the gathered one.
__device__ __forceinline__ uint4 ldg8hc(const uint16_t* p) {
    uint4 r;
    asm("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];" : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
    return r;
}
__device__ __forceinline__ uint4 ldg8h(const uint16_t* p) {
    uint4 r;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "l"(p));
    return r;
}
__device__ __forceinline__ float sqdiff_h2(uint32_t a, uint32_t b, float S) {
    const float2 fa = __half22float2(*reinterpret_cast<const __half2*>(&a));
    const float2 fb = __half22float2(*reinterpret_cast<const __half2*>(&b));
    const float t0 = fa.x - fb.x, t1 = fa.y - fb.y;
    return fmaf(t1, t1, fmaf(t0, t0, S));
}

// Longer rows: a warp takes 32 band pairs; for each pair the lanes stream the
// two rows (coalesced; with VEC = 8, eight values per lane and load when d is
// a multiple of 256 and the rows are 32-byte aligned) and reduce S across the
// warp, and lane p then decides pair p.  With FP16 copies (R.Xh) a first pass
// over them decides almost every pair of a wide band at half the bytes; only
// the pairs it leaves open stream the FP32 rows.
template <int VEC>
__global__ void __launch_bounds__(256) band_recheck_warp_kernel(const double* __restrict__ X,
                                                                uint32_t d,
                                                                const uint32_t* __restrict__ perm,
                                                                double T, Recheck32 R,
                                                                const BandPair* __restrict__ band,
                                                                uint64_t nband, uint64_t n,
                                                                int32_t* counts, DevStatus* st,
                                                                Emit em) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const uint64_t nwarps = (uint64_t)gridDim.x * blockDim.x / 32;
    unsigned hits = 0, exact_runs = 0;
    for (uint64_t base = warp * 32; base < nband; base += nwarps * 32) {
        const uint64_t e = base + lane;
        BandPair bp = {0xffffffffu, 0xffffffffu};
        if (e < nband) bp = band[e];
        const uint32_t mi = bp.i, mj = bp.j & ~kBandBoth;
        const bool valid = e < nband && mi < n && mj < R.nb;
        bool open = valid, hit = false;
        if (R.Xh) {
            float mh = 0.0f;
            for (uint32_t q = 0; q < 32; ++q) {
                const uint32_t i = __shfl_sync(0xffffffffu, mi, q);
                const uint32_t j = __shfl_sync(0xffffffffu, mj, q);
                const bool v = __shfl_sync(0xffffffffu, valid, q);
                if (!v) continue;  // warp-uniform
                const uint16_t* a = R.Xh + (uint64_t)i * d;
                const uint16_t* b = R.Xhb + (uint64_t)j * d;
                float S = 0.0f;
                if (VEC == 8) {
                    for (uint32_t c = 8 * lane; c < d; c += 256) {
                        const uint4 u = ldg8hc(a + c), w = ldg8h(b + c);
                        S = sqdiff_h2(u.x, w.x, S);
                        S = sqdiff_h2(u.y, w.y, S);
                        S = sqdiff_h2(u.z, w.z, S);
                        S = sqdiff_h2(u.w, w.w, S);
                    }
                } else {
                    for (uint32_t c = lane; c < d; c += 32) {
                        const float t = __half2float(__ushort_as_half(a[c])) -
                                        __half2float(__ushort_as_half(b[c]));
                        S = fmaf(t, t, S);
                    }
                }
                for (int o = 16; o; o >>= 1) S += __shfl_xor_sync(0xffffffffu, S, o);
                if (lane == q) mh = S;
            }
            if (valid) {
                const int dec = decide16(R, mi, mj, mh);
                if (dec >= 0) {
                    open = false;
                    hit = dec == 1;
                }
            }
        }
        float mine = 0.0f;
        for (uint32_t left = __ballot_sync(0xffffffffu, open); left; left &= left - 1) {
            const uint32_t q = __ffs(left) - 1;
            const uint32_t i = __shfl_sync(0xffffffffu, mi, q);
            const uint32_t j = __shfl_sync(0xffffffffu, mj, q);
            const float* a = R.Xf + (uint64_t)i * d;
            const float* b = R.Xfb + (uint64_t)j * d;
            float S = 0.0f;
            if (VEC == 8) {
                for (uint32_t c = 8 * lane; c < d; c += 256) {
                    float u[8], w[8];
                    ldg8c(a + c, u);
                    ldg8(b + c, w);
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const float t = u[k] - w[k];
                        S = fmaf(t, t, S);
                    }
                }
            } else {
                for (uint32_t c = lane; c < d; c += 32) {
                    const float t = a[c] - b[c];
                    S = fmaf(t, t, S);
                }
            }
            for (int o = 16; o; o >>= 1) S += __shfl_xor_sync(0xffffffffu, S, o);
            if (lane == q) mine = S;
        }
        if (open) hit = recheck_decide(X, d, perm, T, R, mi, mj, mine, exact_runs);
        if (hit) {
            atomicAdd(&counts[mi], 1);
            if (bp.j & kBandBoth) atomicAdd(&counts[mj], 1);
            emit_pair(em, bp);
            ++hits;
        }
    }
    recheck_totals(st, hits, exact_runs);
}

}  // namespace

static float f32_down(double v) {
    float f = (float)v;
    if ((double)f > v) f = nextafterf(f, -INFINITY);
    return f;
}
static float f32_up(double v) {
    float f = (float)v;
    if ((double)f < v) f = nextafterf(f, INFINITY);
    return f;
}

void finish_recheck32(Recheck32& R) {
    R.f_sTlo = f32_down(R.sTlo);
    R.f_sThi = f32_up(R.sThi);
    // 4 units of FP64 rounding cover the evaluation of 1 -/+ c32 in FP64
    R.f_kin = f32_down((1.0 - R.c32) * (1.0 - 4 * kU));
    R.f_kout = f32_up((1.0 + R.c32) * (1.0 + 4 * kU));
    R.f_abs = f32_up(R.abs32 * (1.0 + 4 * kU));
}

int launch_band_recheck2(const double* X, uint64_t n, uint32_t d, const uint32_t* perm, double T,
                         const Recheck32& R, const BandPair* band, uint64_t nband, int32_t* counts,
                         DevStatus* st, const Emit* em, cudaStream_t s) {
    if (nband == 0) return EJOIN_OK;
    const Emit e = em ? *em : Emit{nullptr, 0, nullptr, 0, nullptr};
    // measured on GB300: a thread per pair wins for rows of <= 256 bytes, a
    // warp per pair (more pairs in flight per load) for longer rows
    const bool thread = d <= 64 && d % 4 == 0 && (((uintptr_t)R.Xf | (uintptr_t)R.Xfb) & 15) == 0;
    if (thread) {
        // 32-byte loads when the rows allow them (half the load instructions)
        const bool v8 = d % 8 == 0 && (((uintptr_t)R.Xf | (uintptr_t)R.Xfb) & 31) == 0;
        const unsigned blocks = (unsigned)std::min<uint64_t>((nband + 255) / 256, 152ull * 32);
        if (v8)
            band_recheck_thread_kernel<true><<<blocks, 256, 0, s>>>(X, d, perm, T, R, band, nband, n, counts, st, e);
        else
            band_recheck_thread_kernel<false><<<blocks, 256, 0, s>>>(X, d, perm, T, R, band, nband, n, counts, st, e);
    } else {
        const uint64_t warps = (nband + 31) / 32;
        const unsigned blocks = (unsigned)std::min<uint64_t>((warps + 7) / 8, 152ull * 64);
        const uintptr_t al = (uintptr_t)R.Xf | (uintptr_t)R.Xfb;
        // 32-byte loads (the streamed row j not allocated in L1) for d a
        // multiple of 256; measured no faster than scalar loads at d = 128
        if (d % 256 == 0 && (al & 31) == 0)
            band_recheck_warp_kernel<8><<<blocks, 256, 0, s>>>(X, d, perm, T, R, band, nband, n, counts, st, e);
        else
            band_recheck_warp_kernel<1><<<blocks, 256, 0, s>>>(X, d, perm, T, R, band, nband, n, counts, st, e);
    }
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

int launch_direct_selfjoin(const double* X, uint64_t n, uint32_t d, double T, int32_t* counts,
                           const Emit* em, cudaStream_t s) {
    if (n == 0) return EJOIN_OK;
    uint64_t nT = (n + TB - 1) / TB;
    uint64_t tiles = nT * (nT + 1) / 2;
    uint64_t gx = tiles < 1048576ull ? tiles : 1048576ull;
    uint64_t gy = (tiles + gx - 1) / gx;
    if (gy > 65535)
        return set_error(EJOIN_EUNSUPPORTED, "direct join: %llu tile pairs exceed the grid",
                         (unsigned long long)tiles);
    const Emit e = em ? *em : Emit{nullptr, 0, nullptr, 0, nullptr};
    direct_selfjoin_kernel<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(X, n, d, T, nT, tiles,
                                                                            counts, e);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

int launch_direct_query(const double* X, uint64_t n, uint32_t d, double T, const uint64_t* rows,
                        uint64_t nq, int32_t* counts, cudaStream_t s, const double* Xq) {
    if (n == 0 || nq == 0) return EJOIN_OK;
    const uint64_t gx = (n + TB - 1) / TB;
    if (gx > 0x7fffffffull) return set_error(EJOIN_EUNSUPPORTED, "query grid too large");
    // the grid's y extent is limited: queries in chunks of 65535 tiles
    const uint64_t chunk = 65535ull * TB;
    for (uint64_t q0 = 0; q0 < nq; q0 += chunk) {
        const uint64_t m = std::min<uint64_t>(chunk, nq - q0);
        direct_query_kernel<<<dim3((unsigned)gx, (unsigned)((m + TB - 1) / TB)), 256, 0, s>>>(
            X, n, d, T, rows ? rows + q0 : nullptr, Xq ? Xq + q0 * (uint64_t)d : nullptr, m,
            counts + q0);
        EJ_CUDA(cudaGetLastError());
        note_launch();
    }
    return EJOIN_OK;
}

int launch_band_recheck(const double* X, uint64_t n, uint32_t d, const uint32_t* perm, double T,
                        const BandPair* band, uint64_t nband, int32_t* counts, DevStatus* st,
                        cudaStream_t s) {
    if (nband == 0) return EJOIN_OK;
    uint64_t blocks = (nband + 255) / 256;
    if (blocks > 0x7fffffffull) return set_error(EJOIN_EUNSUPPORTED, "band too large");
    band_recheck_kernel<<<(unsigned)blocks, 256, 0, s>>>(X, d, perm, T, band, nband, n, counts,
                                                         st);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

}  // namespace ejoin
