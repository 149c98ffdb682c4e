// k_learn.cu -- learned contractive projection and tile-pair pruning.
//
// New relative to the reference (which has no pruning): a k x d FP32
// projection P with ||P||_2 <= sigma (certified) gives the guaranteed lower
// bound  |x_i - x_j| >= |P x_i - P x_j| / sigma.  Points are ordered along the
// projected coordinates (Morton key over the leading coordinates, or the
// leading coordinate alone), the 128-row tiles of that order get bounding
// boxes in projected space (widened by the FP64 rounding bound of each
// projection), and a tile pair whose boxes are farther apart than
// sigma * sqrt(T_hi) cannot hold a neighbour pair: the work-list builder
// (k_misc.cu) drops it before any GEMM.  Skipped tiles contribute 0, which is
// exact because the bound is rigorous.
//
// Training (on the GPU, by this file's kernels):
//   pairs   sampled by the join: half uniform random pairs, half pairs that
//           are close in the current projected order (the pairs that decide
//           whether neighbouring tiles can be skipped); exact FP64 distances
//   forward y = P v (v = x_i - x_j), r = |y|
//   loss    hinge on pairs farther than eps: mean max(0, 1 - r / t),
//           t = min(delta, 2 eps)
//   backward dL/dP = - sum_active (1 / (M t r)) y v^T
//   step    Adam, then power-iteration renormalisation P <- P / max(1, s),
//           s an (inflated) power-iteration estimate of ||P||_2
// The final certificate is ejoin_certify_spectral_norm (host.cpp).
#include <cub/cub.cuh>

#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "ejoin_internal.cuh"

namespace ejoin {

int cert_spectral_norm(const float* P, uint32_t k, uint32_t d, double* out);

namespace {

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// ------------------------------------------------------------ projection --

__device__ __forceinline__ uint32_t ordered_bits32(float v) {
    const uint32_t b = __float_as_uint(v);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float from_ordered_bits32(uint32_t b) {
    b = (b & 0x80000000u) ? (b & 0x7fffffffu) : ~b;
    return __uint_as_float(b);
}

// proj[i][a] = fl32(sum_c P[a][c] Y32[i][c]) (FP32 FMA chain, c in order);
// with Yerr, err[i] bounds |proj[i][a] - P_a (x_i - mu)| for every a:
//   FP32 accumulation of d terms <= (d + 2) 2^-24 sum_c |P_ac| |Y_c|
//                                <= (d + 2) 2^-24 |P_a| |Y|   (Cauchy-Schwarz)
//   centring error               <= |P_a| Yerr_i
// so err = pmax ((d + 4) 2^-24 (1 + 2^-16) |Y| + Yerr_i) + d 2^-148 (rounded
// up), pmax >= max_a |P_a| (host, rounded up).  Projections of x - mu give
// the same differences P(x_i - x_j) as projections of x.  Non-finite rows
// get NaN.  A persistent block stages 128 rows x 64 coordinates at a time in
// shared memory (coalesced loads; row pitch 65: conflict-free), a thread then
// projects one row; the block also folds the per-coordinate range of the
// finite projections into mn / mx (order-preserving bits, one atomic each).
constexpr uint32_t PJ_ROWS = 128, PJ_CH = 64;
template <int K>
__global__ void __launch_bounds__(PJ_ROWS) project_kernel(
    const float* __restrict__ Y32, const float* __restrict__ Yerr, const uint8_t* __restrict__ bad,
    uint64_t n, uint32_t d, const float* __restrict__ P, uint32_t k, float pmax, float* proj,
    float* err, unsigned int* mn, unsigned int* mx) {
    // rows at a pitch of PJ_CH + 4 floats (16-byte aligned rows; a quarter-warp
    // of 16-byte row reads covers all banks once); P transposed [c][a], so
    // each column's K weights are 16-byte broadcast loads
    constexpr uint32_t PITCH = PJ_CH + 4;
    extern __shared__ float4 pj_dyn[];  // two row tiles of PJ_ROWS x PITCH floats
    float* sY = reinterpret_cast<float*>(pj_dyn);
    __shared__ __align__(16) float sP[PJ_CH * K];
    __shared__ unsigned int smn[4][K], smx[4][K];
    const uint32_t t = threadIdx.x, lane = t & 31, w = t >> 5;
    // every chunk is a whole number of float4s when d % 4 == 0 (cw then too)
    const bool vec4 = d % 4 == 0 && (((uintptr_t)Y32) & 15) == 0;
    const float NaNf = __int_as_float(0x7fc00000);
    const float c1 = (float)(d + 4) * 5.9604644775390625e-08f * 1.0000153f;  // (d+4) 2^-24 (1+2^-16)
    uint32_t lo[K], hi[K];
#pragma unroll
    for (int a = 0; a < K; ++a) {
        lo[a] = 0xffffffffu;
        hi[a] = 0u;
    }
    // one row of outputs (and the box bounds) from the accumulated projection
    auto finish_row = [&](uint64_t i, const float (&acc)[K], float s2) {
        if (i >= n) return;
        if (bad[i]) {
            for (uint32_t a = 0; a < k; ++a) proj[i * k + a] = NaNf;
            if (err) err[i] = NaNf;
            return;
        }
#pragma unroll
        for (int a = 0; a < K; ++a)
            if (a < (int)k) {
                proj[i * k + a] = acc[a];
                const uint32_t b = ordered_bits32(acc[a]);
                lo[a] = min(lo[a], b);
                hi[a] = max(hi[a], b);
            }
        if (err) {
            const float inner = __fmaf_ru(c1, __fsqrt_ru(s2), Yerr[i]);
            err[i] = __fmaf_ru(pmax, inner, (float)d * 3.5873240686715317e-43f);
        }
    };
    const uint64_t stride = (uint64_t)gridDim.x * PJ_ROWS;
    if (vec4 && d <= PJ_CH) {
        // rows of at most PJ_CH coordinates: P staged once, row tiles double
        // buffered with cp.async (the next tile's copies run while this one is
        // projected; no registers hold them).  Same arithmetic order as below.
        for (uint32_t e = t; e < K * PJ_CH; e += PJ_ROWS) {
            const uint32_t c = e / K, a = e % K;
            sP[e] = (a < k && c < d) ? P[a * d + c] : 0.0f;
        }
        auto issue = [&](uint64_t i0b, float* dst) {
            for (uint32_t e4 = t; e4 < PJ_ROWS * PJ_CH / 4; e4 += PJ_ROWS) {
                const uint32_t r = e4 / (PJ_CH / 4), c = (e4 % (PJ_CH / 4)) * 4;
                float* q = dst + r * PITCH + c;
                if (i0b + r < n && c < d) {
                    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(q);
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa),
                                 "l"(Y32 + (i0b + r) * d + c));
                } else {
                    *reinterpret_cast<float4*>(q) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                }
            }
            asm volatile("cp.async.commit_group;\n" ::);
        };
        uint32_t buf = 0;
        uint64_t i0 = blockIdx.x * (uint64_t)PJ_ROWS;
        if (i0 < n) issue(i0, sY);
        for (; i0 < n; i0 += stride, buf ^= 1u) {
            const bool more = i0 + stride < n;
            if (more) issue(i0 + stride, sY + (buf ^ 1u) * PJ_ROWS * PITCH);
            if (more) asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            else asm volatile("cp.async.wait_group 0;\n" ::: "memory");
            __syncthreads();
            const float* y = sY + buf * PJ_ROWS * PITCH + t * PITCH;
            float acc[K];
#pragma unroll
            for (int a = 0; a < K; ++a) acc[a] = 0.0f;
            float s2 = 0.0f;
#pragma unroll 2
            for (uint32_t c = 0; c < d; c += 4) {
                const float4 y4 = *reinterpret_cast<const float4*>(y + c);
                const float yv[4] = {y4.x, y4.y, y4.z, y4.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    s2 = __fmaf_ru(yv[u], yv[u], s2);
                    const float4* pp = reinterpret_cast<const float4*>(sP + (c + u) * K);
#pragma unroll
                    for (int a4 = 0; a4 < K / 4; ++a4) {
                        const float4 wv = pp[a4];
                        acc[4 * a4 + 0] = fmaf(wv.x, yv[u], acc[4 * a4 + 0]);
                        acc[4 * a4 + 1] = fmaf(wv.y, yv[u], acc[4 * a4 + 1]);
                        acc[4 * a4 + 2] = fmaf(wv.z, yv[u], acc[4 * a4 + 2]);
                        acc[4 * a4 + 3] = fmaf(wv.w, yv[u], acc[4 * a4 + 3]);
                    }
                }
            }
            finish_row(i0 + t, acc, s2);
            __syncthreads();  // this buffer is refilled two tiles later
        }
    } else
    for (uint64_t i0 = blockIdx.x * (uint64_t)PJ_ROWS; i0 < n; i0 += stride) {
        const uint64_t i = i0 + t;
        float acc[K];
#pragma unroll
        for (int a = 0; a < K; ++a) acc[a] = 0.0f;
        float s2 = 0.0f;
        for (uint32_t c0 = 0; c0 < d; c0 += PJ_CH) {
            const uint32_t cw = min(PJ_CH, d - c0);
            __syncthreads();
            if (vec4) {
                // 16-byte loads, several in flight per thread (rows 16-byte aligned)
#pragma unroll 4
                for (uint32_t e4 = t; e4 < PJ_ROWS * PJ_CH / 4; e4 += PJ_ROWS) {
                    const uint32_t r = e4 / (PJ_CH / 4), c = (e4 % (PJ_CH / 4)) * 4;
                    float4 v4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (i0 + r < n && c < cw)
                        v4 = __ldg(reinterpret_cast<const float4*>(Y32 + (i0 + r) * d + c0 + c));
                    *reinterpret_cast<float4*>(sY + r * PITCH + c) = v4;
                }
            } else {
                for (uint32_t e = t; e < PJ_ROWS * PJ_CH; e += PJ_ROWS) {
                    const uint32_t r = e / PJ_CH, c = e % PJ_CH;
                    sY[r * PITCH + c] = (i0 + r < n && c < cw) ? Y32[(i0 + r) * d + c0 + c] : 0.0f;
                }
            }
            for (uint32_t e = t; e < K * PJ_CH; e += PJ_ROWS) {
                const uint32_t c = e / K, a = e % K;
                sP[e] = (a < k && c < cw) ? P[a * d + c0 + c] : 0.0f;
            }
            __syncthreads();
            // four columns per step (columns past cw hold zeros in sY and sP)
            const float* y = sY + t * PITCH;
#pragma unroll 2
            for (uint32_t c = 0; c < cw; c += 4) {
                const float4 y4 = *reinterpret_cast<const float4*>(y + c);
                const float yv[4] = {y4.x, y4.y, y4.z, y4.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    s2 = __fmaf_ru(yv[u], yv[u], s2);
                    const float4* pp = reinterpret_cast<const float4*>(sP + (c + u) * K);
#pragma unroll
                    for (int a4 = 0; a4 < K / 4; ++a4) {
                        const float4 wv = pp[a4];
                        acc[4 * a4 + 0] = fmaf(wv.x, yv[u], acc[4 * a4 + 0]);
                        acc[4 * a4 + 1] = fmaf(wv.y, yv[u], acc[4 * a4 + 1]);
                        acc[4 * a4 + 2] = fmaf(wv.z, yv[u], acc[4 * a4 + 2]);
                        acc[4 * a4 + 3] = fmaf(wv.w, yv[u], acc[4 * a4 + 3]);
                    }
                }
            }
        }
        finish_row(i, acc, s2);
    }
#pragma unroll
    for (int a = 0; a < K; ++a)
        for (int o = 16; o; o >>= 1) {
            lo[a] = min(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = max(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    if (lane == 0)
#pragma unroll
        for (int a = 0; a < K; ++a) {
            smn[w][a] = lo[a];
            smx[w][a] = hi[a];
        }
    __syncthreads();
    if (t < k) {
        uint32_t l = smn[0][t], h = smx[0][t];
        for (int q = 1; q < (int)(PJ_ROWS / 32); ++q) {
            l = min(l, smn[q][t]);
            h = max(h, smx[q][t]);
        }
        if (l != 0xffffffffu) atomicMin(&mn[t], l);
        if (h != 0u) atomicMax(&mx[t], h);
    }
}

// Sort keys: Morton interleave of the leading min(k, 8) coordinates quantised
// to 64 / m bits each, or the order-preserving bits of coordinate 0.  NaN
// rows sort last.  The quantisation (v - lo) * (levels / span) in FP32 is
// monotone in v, which is all the ordering needs.
__global__ void key_kernel(const float* __restrict__ proj, uint64_t n, uint32_t k, int lead_only,
                           const unsigned int* mn, const unsigned int* mx,
                           unsigned long long* keys, uint32_t* idx) {
    const uint32_t m = k < 8 ? k : 8;
    const uint32_t bits = 64 / m;
    const uint32_t qb = bits > 31 ? 31 : bits;
    const uint32_t qmax = (1u << qb) - 1u;
    __shared__ float slo[8], sinv[8];
    if (threadIdx.x < m) {
        const float lo = from_ordered_bits32(mn[threadIdx.x]);
        const float hi = from_ordered_bits32(mx[threadIdx.x]);
        const float span = hi - lo;
        slo[threadIdx.x] = lo;
        sinv[threadIdx.x] = span > 0.0f ? (float)qmax / span : 0.0f;
    }
    __syncthreads();
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    idx[i] = (uint32_t)i;
    const float p0 = proj[i * k];
    if (isnan(p0)) {
        keys[i] = ~0ull;
        return;
    }
    if (lead_only) {
        keys[i] = ordered_bits32(p0);
        return;
    }
    uint32_t q[8];
#pragma unroll
    for (uint32_t a = 0; a < 8; ++a) {
        q[a] = 0;
        if (a < m) {
            const float t = fmaxf((proj[i * k + a] - slo[a]) * sinv[a], 0.0f);  // NaN -> 0
            q[a] = min(__float2uint_rz(t), qmax);
        }
    }
    unsigned long long key = 0;
    for (int b = (int)qb - 1; b >= 0; --b)
        for (uint32_t a = 0; a < m; ++a) key = (key << 1) | ((q[a] >> b) & 1u);
    keys[i] = key;
}

// Per 128-row tile of the sorted order: [lo, hi] of every projected
// coordinate, widened by each row's error bound (outward rounding);
// non-finite and padding rows are left out (they are never neighbours).
// A thread per row reads its row's K projections with 16-byte loads (one
// gathered row instead of K scattered words), then warps and the block
// reduce the bounds (min / max are exact in any order).
template <int K>
__global__ void __launch_bounds__(128) boxes_kernel(const float* __restrict__ proj,
                                                    const float* __restrict__ err,
                                                    const uint32_t* __restrict__ perm, uint64_t n,
                                                    uint32_t k, float* lo, float* hi) {
    __shared__ float sl[4][K], sh[4][K];
    const uint64_t t = blockIdx.x;
    const uint32_t r = threadIdx.x, lane = r & 31, w = r >> 5;
    float l[K], h[K];
#pragma unroll
    for (int a = 0; a < K; ++a) {
        l[a] = INFINITY;
        h[a] = -INFINITY;
    }
    const uint64_t p = t * 128 + r;
    if (p < n) {
        const uint64_t i = perm[p];
        const float e = err[i];
        float v[K];
        if (k == (uint32_t)K) {
            const float4* src = reinterpret_cast<const float4*>(proj + i * K);
#pragma unroll
            for (int a4 = 0; a4 < K / 4; ++a4) {
                const float4 q = __ldg(&src[a4]);
                v[4 * a4 + 0] = q.x;
                v[4 * a4 + 1] = q.y;
                v[4 * a4 + 2] = q.z;
                v[4 * a4 + 3] = q.w;
            }
        } else {
#pragma unroll
            for (int a = 0; a < K; ++a) v[a] = a < (int)k ? proj[i * k + a] : 0.0f;
        }
        if (!isnan(e)) {
#pragma unroll
            for (int a = 0; a < K; ++a)
                if (a < (int)k && !isnan(v[a])) {
                    l[a] = __fsub_rd(v[a], e);
                    h[a] = __fadd_ru(v[a], e);
                }
        }
    }
#pragma unroll
    for (int a = 0; a < K; ++a)
        for (int o = 16; o; o >>= 1) {
            l[a] = fminf(l[a], __shfl_xor_sync(0xffffffffu, l[a], o));
            h[a] = fmaxf(h[a], __shfl_xor_sync(0xffffffffu, h[a], o));
        }
    if (lane == 0) {
#pragma unroll
        for (int a = 0; a < K; ++a) {
            sl[w][a] = l[a];
            sh[w][a] = h[a];
        }
    }
    __syncthreads();
    if (r < k) {
        lo[t * k + r] = fminf(fminf(sl[0][r], sl[1][r]), fminf(sl[2][r], sl[3][r]));
        hi[t * k + r] = fmaxf(fmaxf(sh[0][r], sh[1][r]), fmaxf(sh[2][r], sh[3][r]));
    }
}

// Boxes of super-blocks of `sb` consecutive tiles (union of the tile boxes).
__global__ void superbox_kernel(const float* __restrict__ lo, const float* __restrict__ hi,
                                uint64_t nt, uint32_t k, uint32_t sb, float* slo, float* shi) {
    const uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t ns = (nt + sb - 1) / sb;
    if (e >= ns * k) return;
    const uint64_t S = e / k;
    const uint32_t a = (uint32_t)(e % k);
    float l = INFINITY, h = -INFINITY;
    for (uint64_t t = S * sb; t < min(nt, (S + 1) * sb); ++t) {
        l = fminf(l, lo[t * k + a]);
        h = fmaxf(h, hi[t * k + a]);
    }
    slo[e] = l;
    shi[e] = h;
}

// --------------------------------------------------------------- training --

struct PairBatch {
    float* V;        // [M][d] differences (FP32; training does not need exactness)
    float* tgt;      // [M] hinge target t (0 = pair not far: inactive)
};

// Half uniform random pairs, half pairs close in the current order (perm);
// differences and distances from the FP32 centred copy (training needs no
// exactness).  Pairs with a non-finite row are inactive.  A group of 8 lanes
// builds one pair (16-byte loads when d % 4 == 0), so a warp has 4 pairs in
// flight.
__global__ void sample_pairs_kernel(const float* __restrict__ Y32, const uint8_t* __restrict__ bad,
                                    uint64_t n, uint32_t d, const uint32_t* __restrict__ perm,
                                    uint64_t M, uint64_t seed, double eps, uint32_t window,
                                    PairBatch pb) {
    constexpr uint32_t G = 8;
    const uint32_t lane = threadIdx.x & 31, g = lane % G;
    const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    const float lo = (float)(eps * 1.02), cap = (float)(2.0 * eps);
    const bool v4 = d % 4 == 0 && (((uintptr_t)Y32 | (uintptr_t)pb.V) & 15) == 0;
    for (uint64_t base = gw * (32 / G); base < M; base += nw * (32 / G)) {  // warp-uniform
        const uint64_t e = base + lane / G;
        const bool act = e < M;
        uint64_t i = 0, j = 0;
        if (act) {
            // indices by multiply-high reduction of the hashes (no 64-bit
            // division, which the GPU emulates in software)
            const uint64_t h1 = splitmix64(seed ^ (e * 0x9E3779B97F4A7C15ull));
            const uint64_t h2 = splitmix64(h1);
            if (e & 1) {
                i = __umul64hi(h1, n);
                j = __umul64hi(h2, n);
            } else {
                const uint64_t t = __umul64hi(h1, n);
                const uint64_t off = 1 + (uint32_t)h2 % window;
                uint64_t u = t + off;
                if (u >= n) u = t >= off ? t - off : 0;
                i = perm ? perm[t] : t;
                j = perm ? perm[u] : u;
            }
        }
        float s = 0.0f;
        if (act) {
            const float* a = Y32 + i * d;
            const float* b = Y32 + j * d;
            float* v = pb.V + e * d;
            if (v4) {
#pragma unroll 2
                for (uint32_t c = g; c < d / 4; c += G) {
                    const float4 x = __ldg(reinterpret_cast<const float4*>(a) + c);
                    const float4 y = __ldg(reinterpret_cast<const float4*>(b) + c);
                    const float4 t = make_float4(x.x - y.x, x.y - y.y, x.z - y.z, x.w - y.w);
                    s = fmaf(t.x, t.x, fmaf(t.y, t.y, fmaf(t.z, t.z, fmaf(t.w, t.w, s))));
                    reinterpret_cast<float4*>(v)[c] = t;
                }
            } else {
                for (uint32_t c = g; c < d; c += G) {
                    const float t = a[c] - b[c];
                    s = fmaf(t, t, s);
                    v[c] = t;
                }
            }
        }
#pragma unroll
        for (uint32_t o = G / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (act && g == 0) {
            const float delta = sqrtf(s);
            float t = 0.0f;
            if (!bad[i] && !bad[j] && delta > lo) t = fminf(delta, cap);
            pb.tgt[e] = t;
        }
    }
}

constexpr int TRAIN_THREADS = 256;

// Pairs per shared-memory tile of the training kernel.
__host__ __device__ inline uint32_t train_tile_pairs(uint32_t d) {
    uint32_t tp = 16384u / d;
    tp = tp > 256u ? 256u : tp;
    return tp < 8u ? 8u : tp;
}
// Shared memory of train_step_kernel<K>: P transposed [d][K], the block's
// gradient [K][d], the pair tile [TP][d + 1] (rounded up to whole float4s, so
// that the coefficients start 16-byte aligned), the coefficients [TP][K].
__host__ __device__ inline uint32_t train_tile_floats(uint32_t d) {
    return (train_tile_pairs(d) * (d + 1) + 3u) & ~3u;
}
__host__ inline size_t train_smem_bytes(uint32_t k, uint32_t d) {
    const uint32_t K = k <= 8 ? 8 : 16;
    const uint32_t tp = train_tile_pairs(d);
    return (size_t)(2 * K * d + train_tile_floats(d) + tp * K) * sizeof(float);
}
// Pair slices of the backward pass: Q threads share a column c, each summing
// every Q-th pair of the tile (their partials fit in the pair tile's space).
__host__ __device__ inline uint32_t train_slices(uint32_t d, uint32_t K) {
    const uint32_t tp = train_tile_pairs(d);
    uint32_t q = d >= TRAIN_THREADS ? 1u : TRAIN_THREADS / d;
    const uint32_t cap = tp * (d + 1) / (K * d);
    q = q < cap ? q : cap;
    return q < 1u ? 1u : q;
}

// Gradient and loss are accumulated in 64-bit fixed point (2^-40 units)
// with integer atomics: integer addition is associative, so the result does
// not depend on the order in which blocks finish (bit-reproducible training).
constexpr double kFix = 1099511627776.0;  // 2^40
// v * 2^40 is exact in FP32 as in FP64, so the FP32 conversion gives the same
// integer (FP64 arithmetic is slow on GB300)
__device__ __forceinline__ void fix_add(unsigned long long* dst, float v) {
    atomicAdd(dst, (unsigned long long)__float2ll_rn(v * 1099511627776.0f));
}
// integer / 2^40 as FP32: one rounding (int64 -> FP32), then an exact scaling
__device__ __forceinline__ float fix_value(unsigned long long g) {
    return __ll2float_rn((long long)g) * 9.094947017729282379e-13f;
}

// One Adam step on P from G (G is cleared for the next step), then the
// power-iteration renormalisation P <- P / max(1, 1.02 s): s is the Rayleigh
// quotient estimate of ||P||_2 from (P P^T)^32 (five normalised squarings, so
// it converges when the leading eigenvalues are close).  One block; k <= 16;
// P is kept in shared memory (sPa: k * d floats) between the phases.  Run by
// one whole block (blockDim.x a multiple of 32): the separate kernel below,
// or the last block of train_step_kernel.
__device__ void adam_renorm_block(float* P, unsigned long long* G, float* m1, float* m2,
                                  uint32_t k, uint32_t d, float lr, float b1, float b2, float c1,
                                  float c2, int renorm, float* sigma_out, float* sPa) {
    __shared__ float M[16 * 16], A[16 * 16], B[16 * 16];
    __shared__ float v[16];
    __shared__ float lam;
    const uint32_t nel = k * d;
    for (uint32_t e = threadIdx.x; e < nel; e += blockDim.x) {
        const float g = fix_value(__ldcg(&G[e]));  // L2: other blocks added it
        G[e] = 0ull;
        const float a = b1 * m1[e] + (1.0f - b1) * g;
        const float b = b2 * m2[e] + (1.0f - b2) * g * g;
        m1[e] = a;
        m2[e] = b;
        const float pv = P[e] - lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
        sPa[e] = pv;
        if (!renorm) P[e] = pv;
    }
    if (!renorm) return;
    __syncthreads();
    // M = P P^T: warp per entry
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x / 32, nw = blockDim.x / 32;
    for (uint32_t e = wid; e < k * k; e += nw) {
        const uint32_t a = e / k, b = e % k;
        float s = 0.0f;
        for (uint32_t c = lane; c < d; c += 32) s = fmaf(sPa[a * d + c], sPa[b * d + c], s);
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            M[e] = s;
            A[e] = s;
        }
    }
    // the k x k part runs in warp 0 (warp-level synchronisation only): five
    // normalised squarings, 8 power-iteration steps, the Rayleigh quotient
    if (wid == 0) {
        const uint32_t kk = k * k;
        for (int sq = 0; sq < 5; ++sq) {
            float mx = 0.0f;
            for (uint32_t e = lane; e < kk; e += 32) mx = fmaxf(mx, fabsf(A[e]));
            for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            const float inv = mx > 0.0f ? 1.0f / mx : 0.0f;
            for (uint32_t e = lane; e < kk; e += 32) {
                const uint32_t a = e / k, b = e % k;
                float s = 0.0f;
                for (uint32_t c = 0; c < k; ++c) s = fmaf(A[a * k + c] * inv, A[c * k + b] * inv, s);
                B[e] = s;
            }
            __syncwarp();
            for (uint32_t e = lane; e < kk; e += 32) A[e] = B[e];
            __syncwarp();
        }
        float vl = lane < k ? 1.0f + 0.01f * lane : 0.0f;  // lane a holds v[a]
        for (int it = 0; it < 8; ++it) {
            if (lane < k) v[lane] = vl;
            __syncwarp();
            float s = 0.0f;
            if (lane < k)
                for (uint32_t b = 0; b < k; ++b) s = fmaf(A[lane * k + b], v[b], s);
            float nn = s * s;
            for (int o = 16; o; o >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, o);
            vl = nn > 0.0f ? s * rsqrtf(nn) : 0.0f;
            __syncwarp();
        }
        if (lane < k) v[lane] = vl;
        __syncwarp();
        float num = 0.0f, den = 0.0f;
        if (lane < k) {
            float s = 0.0f;
            for (uint32_t b = 0; b < k; ++b) s = fmaf(M[lane * k + b], v[b], s);
            num = vl * s;
            den = vl * vl;
        }
        for (int o = 16; o; o >>= 1) {
            num += __shfl_xor_sync(0xffffffffu, num, o);
            den += __shfl_xor_sync(0xffffffffu, den, o);
        }
        if (lane == 0) lam = den > 0.0f ? num / den : 0.0f;
    }
    __syncthreads();
    const float sig = sqrtf(fmaxf(lam, 0.0f)) * 1.02f;
    const float scale = sig > 1.0f ? 1.0f / sig : 1.0f;
    for (uint32_t e = threadIdx.x; e < nel; e += blockDim.x) P[e] = sPa[e] * scale;
    if (threadIdx.x == 0 && sigma_out) *sigma_out = sig;
}

__global__ void adam_renorm_kernel(float* P, unsigned long long* G, float* m1, float* m2,
                                   uint32_t k, uint32_t d, float lr, float b1, float b2, float c1,
                                   float c2, int renorm, float* sigma_out) {
    extern __shared__ float sPa[];  // k * d
    adam_renorm_block(P, G, m1, m2, k, d, lr, b1, b2, c1, c2, renorm, sigma_out, sPa);
}

// Adam state of a training step fused into train_step_kernel (done == null:
// gradient only).
struct AdamArgs {
    float* m1;
    float* m2;
    float lr, b1, b2, c1, c2;
    unsigned int* done;  // blocks finished (reset by the last one)
};

// Forward + hinge loss + backward for M pairs; G += dL/dP, loss += sum of
// hinge terms / M (fixed-point accumulators).  A tile of TP pairs is staged
// once in shared memory (row pitch d + 1: conflict-free) and serves
//   forward   thread per pair (warp per pair for d > 256); P is held
//             transposed, so every coordinate reads its K weights with 16-byte
//             broadcast loads;
//   backward  Q threads per column c, each with K accumulators over every
//             Q-th pair; the Q partials are then added in a fixed order.
template <int K>
__global__ void __launch_bounds__(TRAIN_THREADS) train_step_kernel(float* P, uint32_t k,
                                                                   uint32_t d, PairBatch pb,
                                                                   uint64_t M, AdamArgs ad,
                                                                   unsigned long long* G,
                                                                   unsigned long long* loss) {
    extern __shared__ float4 sm4[];
    float* sm = reinterpret_cast<float*>(sm4);
    const uint32_t TP = train_tile_pairs(d);
    const uint32_t pitch = d + 1;
    const uint32_t Q = train_slices(d, K);
    // P transposed as K/4 planes of float4 (plane a4, column c: rows 4 a4 ..
    // 4 a4 + 3 of column c), zero beyond k: lanes that read different columns
    // (warp per pair) hit consecutive 16-byte words, conflict-free, and
    // threads that read one column (thread per pair) get a broadcast
    float* sPT = sm;
    float* sG = sPT + K * d;       // K * d: this block's gradient partial
    float* sV = sG + K * d;        // TP * pitch (also the backward partials)
    float* sC = sV + train_tile_floats(d);  // TP * K coefficients (16-byte aligned)
    for (uint32_t e = threadIdx.x; e < K * d; e += blockDim.x) {
        const uint32_t t = e / 4, c = t % d, a = 4 * (t / d) + e % 4;
        sPT[e] = a < k ? P[a * d + c] : 0.0f;
        sG[e] = 0.0f;
    }
    const float4* sPT4 = reinterpret_cast<const float4*>(sPT);
    const float invM = 1.0f / (float)M;
    float lsum = 0.0f;
    for (uint64_t base = blockIdx.x * (uint64_t)TP; base < M; base += (uint64_t)gridDim.x * TP) {
        const uint32_t np = (M - base) < TP ? (uint32_t)(M - base) : TP;
        __syncthreads();
        {
            // 16-byte loads, up to sixteen in flight per thread (tile starts are 16-byte
            // aligned: base is a multiple of TP, itself a multiple of 4 or d is)
            const float* src = pb.V + base * d;
            const uint32_t ne = np * d;
            const bool al = (((uintptr_t)src) & 15) == 0;
            const uint32_t n4 = al ? ne / 4 : 0;
            const float4* src4 = reinterpret_cast<const float4*>(src);
#pragma unroll 16
            for (uint32_t e4 = threadIdx.x; e4 < n4; e4 += blockDim.x) {
                const float4 v4 = __ldg(&src4[e4]);
                const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
                uint32_t e = e4 * 4, r = e / d, c = e - r * d;
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    sV[r * pitch + c] = vv[t];
                    if (++c == d) {
                        c = 0;
                        ++r;
                    }
                }
            }
            for (uint32_t e = n4 * 4 + threadIdx.x; e < ne; e += blockDim.x)
                sV[(e / d) * pitch + e % d] = src[e];
        }
        __syncthreads();
        if (d <= 256) {
            // thread per pair
            for (uint32_t p = threadIdx.x; p < TP; p += blockDim.x) {
                float y[K];
#pragma unroll
                for (int a = 0; a < K; ++a) y[a] = 0.0f;
                float coef = 0.0f;
                if (p < np && pb.tgt[base + p] > 0.0f) {
                    const float* v = sV + p * pitch;
                    for (uint32_t c = 0; c < d; ++c) {
                        const float vc = v[c];
#pragma unroll
                        for (int a4 = 0; a4 < K / 4; ++a4) {
                            const float4 w = sPT4[a4 * d + c];
                            y[4 * a4 + 0] = fmaf(w.x, vc, y[4 * a4 + 0]);
                            y[4 * a4 + 1] = fmaf(w.y, vc, y[4 * a4 + 1]);
                            y[4 * a4 + 2] = fmaf(w.z, vc, y[4 * a4 + 2]);
                            y[4 * a4 + 3] = fmaf(w.w, vc, y[4 * a4 + 3]);
                        }
                    }
                    float r2 = 0.0f;
#pragma unroll
                    for (int a = 0; a < K; ++a) r2 = fmaf(y[a], y[a], r2);
                    const float r = sqrtf(r2), t = pb.tgt[base + p];
                    if (r < t) {
                        lsum += 1.0f - r / t;
                        coef = r > 0.0f ? -invM / (t * r) : 0.0f;
                    }
                }
#pragma unroll
                for (int a = 0; a < K; ++a) sC[p * K + a] = coef * y[a];
            }
        } else {
            // warp per pair, lanes over coordinates (large d, few pairs per tile)
            const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x / 32, nw = blockDim.x / 32;
            for (uint32_t p = wid; p < TP; p += nw) {
                const bool act = p < np && pb.tgt[base + p] > 0.0f;  // warp-uniform
                float y[K];
#pragma unroll
                for (int a = 0; a < K; ++a) y[a] = 0.0f;
                if (act) {
                    const float* v = sV + p * pitch;
                    for (uint32_t c = lane; c < d; c += 32) {
                        const float vc = v[c];
#pragma unroll
                        for (int a4 = 0; a4 < K / 4; ++a4) {
                            const float4 w = sPT4[a4 * d + c];
                            y[4 * a4 + 0] = fmaf(w.x, vc, y[4 * a4 + 0]);
                            y[4 * a4 + 1] = fmaf(w.y, vc, y[4 * a4 + 1]);
                            y[4 * a4 + 2] = fmaf(w.z, vc, y[4 * a4 + 2]);
                            y[4 * a4 + 3] = fmaf(w.w, vc, y[4 * a4 + 3]);
                        }
                    }
#pragma unroll
                    for (int a = 0; a < K; ++a)
                        for (int o = 16; o; o >>= 1) y[a] += __shfl_xor_sync(0xffffffffu, y[a], o);
                }
                float coef = 0.0f;
                if (act) {
                    float r2 = 0.0f;
#pragma unroll
                    for (int a = 0; a < K; ++a) r2 = fmaf(y[a], y[a], r2);
                    const float r = sqrtf(r2), t = pb.tgt[base + p];
                    if (r < t) {
                        if (lane == 0) lsum += 1.0f - r / t;
                        coef = r > 0.0f ? -invM / (t * r) : 0.0f;
                    }
                }
                if (lane == 0) {
#pragma unroll
                    for (int a = 0; a < K; ++a) sC[p * K + a] = coef * y[a];
                }
            }
        }
        __syncthreads();
        // G[a][c] += sum_p sC[p][a] * V[p][c]
        if (Q == 1) {
            for (uint32_t c = threadIdx.x; c < d; c += blockDim.x) {
                float acc[K];
#pragma unroll
                for (int a = 0; a < K; ++a) acc[a] = 0.0f;
                for (uint32_t p = 0; p < np; ++p) {
                    const float v = sV[p * pitch + c];
                    const float4* cp = reinterpret_cast<const float4*>(sC + p * K);
#pragma unroll
                    for (int a4 = 0; a4 < K / 4; ++a4) {
                        const float4 w = cp[a4];
                        acc[4 * a4 + 0] = fmaf(w.x, v, acc[4 * a4 + 0]);
                        acc[4 * a4 + 1] = fmaf(w.y, v, acc[4 * a4 + 1]);
                        acc[4 * a4 + 2] = fmaf(w.z, v, acc[4 * a4 + 2]);
                        acc[4 * a4 + 3] = fmaf(w.w, v, acc[4 * a4 + 3]);
                    }
                }
#pragma unroll
                for (int a = 0; a < K; ++a) sG[a * d + c] += acc[a];
            }
        } else {
            const bool own = threadIdx.x < d * Q;
            const uint32_t c = threadIdx.x % d, q = threadIdx.x / d;
            float acc[K];
#pragma unroll
            for (int a = 0; a < K; ++a) acc[a] = 0.0f;
            if (own) {
                for (uint32_t p = q; p < np; p += Q) {
                    const float v = sV[p * pitch + c];
                    const float4* cp = reinterpret_cast<const float4*>(sC + p * K);
#pragma unroll
                    for (int a4 = 0; a4 < K / 4; ++a4) {
                        const float4 w = cp[a4];
                        acc[4 * a4 + 0] = fmaf(w.x, v, acc[4 * a4 + 0]);
                        acc[4 * a4 + 1] = fmaf(w.y, v, acc[4 * a4 + 1]);
                        acc[4 * a4 + 2] = fmaf(w.z, v, acc[4 * a4 + 2]);
                        acc[4 * a4 + 3] = fmaf(w.w, v, acc[4 * a4 + 3]);
                    }
                }
            }
            __syncthreads();  // the pair tile is free: it holds the partials now
            float* red = sV;  // [Q][K][d]
            if (own) {
#pragma unroll
                for (int a = 0; a < K; ++a) red[(q * K + a) * d + c] = acc[a];
            }
            __syncthreads();
            for (uint32_t el = threadIdx.x; el < K * d; el += blockDim.x) {
                float t = 0.0f;
                for (uint32_t qq = 0; qq < Q; ++qq) t += red[qq * K * d + el];
                sG[el] += t;
            }
        }
    }
    __syncthreads();
    for (uint32_t el = threadIdx.x; el < k * d; el += blockDim.x)
        if (sG[el] != 0.0f) fix_add(&G[el], sG[el]);
    for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((threadIdx.x & 31) == 0 && lsum != 0.0f) fix_add(loss, lsum * invM);
    if (!ad.done) return;
    // the last block to finish runs the Adam step and the renormalisation
    // (every block has read P; the gradient atomics are complete once the
    // counter shows all blocks); sPT (K * d floats) is free for P
    __shared__ unsigned s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(ad.done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    adam_renorm_block(P, G, ad.m1, ad.m2, k, d, ad.lr, ad.b1, ad.b2, ad.c1, ad.c2, 1, nullptr, sPT);
    if (threadIdx.x == 0) *ad.done = 0u;
}


}  // namespace

// ------------------------------------------------------------ host side --

// Projects all points with P (device k x d), orders them and, when `boxes` is
// given, computes the boxes of the 128-row tiles and of super-blocks of
// kSuperTiles tiles (FP32, outward rounded).  perm: sorted position ->
// original row.
int learned_order(const float* Y32, const float* Yerr, const uint8_t* bad, uint64_t n,
                  uint64_t n_pad, uint32_t d, const float* P_dev, uint32_t k, float pmax,
                  int lead_only, DBuf<uint32_t>& perm, LearnedBoxes* boxes, cudaStream_t s) {
    if (boxes && !Yerr) return set_error(EJOIN_EINTERNAL, "learned_order: boxes need Yerr");
    DBuf<float> proj, err;
    EJ_TRY(proj.alloc(n * k, s, "projections"));
    if (boxes) EJ_TRY(err.alloc(n, s, "projection error bounds"));
    DBuf<unsigned int> rng;
    EJ_TRY(rng.alloc(2 * k, s, "projection ranges"));
    EJ_CUDA(cudaMemsetAsync(rng.p, 0xff, k * sizeof(unsigned int), s));
    EJ_CUDA(cudaMemsetAsync(rng.p + k, 0, k * sizeof(unsigned int), s));
    {
        int sms = 0, dev = 0;
        EJ_CUDA(cudaGetDevice(&dev));
        EJ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        auto fn = k <= 8 ? project_kernel<8> : project_kernel<16>;
        const size_t dsm = 2 * (size_t)PJ_ROWS * (PJ_CH + 4) * sizeof(float);  // two row tiles
        EJ_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm));
        int per_sm = 0;
        EJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, PJ_ROWS, dsm));
        const uint64_t tiles = (n + PJ_ROWS - 1) / PJ_ROWS;
        const unsigned grid = (unsigned)std::max<uint64_t>(
            1, std::min<uint64_t>(tiles, (uint64_t)sms * std::max(per_sm, 1)));
        fn<<<grid, PJ_ROWS, dsm, s>>>(Y32, boxes ? Yerr : nullptr, bad, n, d, P_dev, k, pmax, proj.p,
                                    boxes ? err.p : nullptr, rng.p, rng.p + k);
        EJ_CUDA(cudaGetLastError());
        note_launch();
    }
    DBuf<unsigned long long> keys, keys2;
    DBuf<uint32_t> idx;
    EJ_TRY(keys.alloc(n, s, "sort keys"));
    EJ_TRY(keys2.alloc(n, s, "sorted keys"));
    EJ_TRY(idx.alloc(n, s, "sort values"));
    EJ_TRY(perm.alloc(n, s, "permutation"));
    key_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(proj.p, n, k, lead_only, rng.p,
                                                           rng.p + k, keys.p, idx.p);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    // Lead-coordinate keys live in bits 0..31.  Morton keys use all 64 bits for
    // the pruning order; the training rounds (no boxes) only need locality for
    // pair sampling and sort on the coarse top 32 bits (half the passes).
    const int b0 = lead_only ? 0 : (boxes ? 0 : 32), b1 = lead_only ? 32 : 64;
    size_t tmp_bytes = 0;
    EJ_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.p, keys2.p, idx.p, perm.p,
                                            (int)n, b0, b1, s));
    DBuf<uint8_t> tmp;
    EJ_TRY(tmp.alloc(tmp_bytes, s, "sort scratch"));
    EJ_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys.p, keys2.p, idx.p, perm.p,
                                            (int)n, b0, b1, s));
    note_launch(b1 - b0 == 64 ? 11 : 7);  // histogram, scan and one-sweep passes of the library sort
    if (boxes) {
        const uint64_t nt = n_pad / 128;
        const uint64_t ns = (nt + kSuperTiles - 1) / kSuperTiles;
        EJ_TRY(boxes->lo.alloc(nt * k, s, "tile boxes"));
        EJ_TRY(boxes->hi.alloc(nt * k, s, "tile boxes"));
        EJ_TRY(boxes->slo.alloc(ns * k, s, "super-block boxes"));
        EJ_TRY(boxes->shi.alloc(ns * k, s, "super-block boxes"));
        if (k <= 8)
            boxes_kernel<8><<<(unsigned)nt, 128, 0, s>>>(proj.p, err.p, perm.p, n, k, boxes->lo.p,
                                                         boxes->hi.p);
        else
            boxes_kernel<16><<<(unsigned)nt, 128, 0, s>>>(proj.p, err.p, perm.p, n, k, boxes->lo.p,
                                                          boxes->hi.p);
        EJ_CUDA(cudaGetLastError());
        superbox_kernel<<<(unsigned)((ns * k + 255) / 256), 256, 0, s>>>(
            boxes->lo.p, boxes->hi.p, nt, k, kSuperTiles, boxes->slo.p, boxes->shi.p);
        EJ_CUDA(cudaGetLastError());
        note_launch(2);
        boxes->k = k;
    }
    return EJOIN_OK;
}

int train_projection_dev(const float* Y32, const uint8_t* bad, uint64_t n, uint32_t d, double eps,
                         uint32_t k, uint64_t pairs, uint32_t steps, uint64_t seed, int lead_only,
                         cudaStream_t s, TrainResult& out) {
    if (k == 0 || k > 16) return set_error(EJOIN_EINVAL, "proj_k must be in 1..16");
    if (n < 2) return set_error(EJOIN_EINVAL, "training needs at least 2 points");
    const uint32_t nel = k * d;
    // seeded Gaussian initialisation (Box-Muller on splitmix64), certified scaling
    std::vector<float> P0(nel);
    for (uint32_t e = 0; e < nel; ++e) {
        const uint64_t a = splitmix64(seed * 0x2545F4914F6CDD1Dull + 2 * e);
        const uint64_t b = splitmix64(seed * 0x2545F4914F6CDD1Dull + 2 * e + 1);
        const double u1 = ((a >> 11) + 1.0) * (1.0 / 9007199254740993.0);
        const double u2 = (b >> 11) * (1.0 / 9007199254740992.0);
        P0[e] = (float)(sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
    }
    double s0 = 0;
    EJ_TRY(cert_spectral_norm(P0.data(), k, d, &s0));
    for (auto& v : P0) v = (float)(v / (s0 * 1.0001));
    DBuf<float> P, m1, m2;
    DBuf<unsigned long long> G, loss;
    EJ_TRY(P.alloc(nel, s, "projection"));
    EJ_TRY(G.alloc(nel, s, "gradient"));
    EJ_TRY(m1.alloc(nel, s, "adam m"));
    EJ_TRY(m2.alloc(nel, s, "adam v"));
    EJ_TRY(loss.alloc(steps + 1, s, "loss"));
    EJ_CUDA(cudaMemcpyAsync(P.p, P0.data(), nel * sizeof(float), cudaMemcpyHostToDevice, s));
    EJ_TRY(G.zero(s));
    EJ_TRY(m1.zero(s));
    EJ_TRY(m2.zero(s));
    EJ_TRY(loss.zero(s));
    DBuf<unsigned int> done;  // blocks finished per step (the fused Adam step)
    EJ_TRY(done.alloc(1, s, "step counter"));
    EJ_TRY(done.zero(s));
    const uint64_t M = std::max<uint64_t>(pairs ? pairs : (1u << 19), 256);
    const uint64_t B = std::min<uint64_t>(M, 65536);  // minibatch
    DBuf<float> V, tgt;
    EJ_TRY(V.alloc(M * d, s, "training pair differences"));
    EJ_TRY(tgt.alloc(M, s, "training pair targets"));
    const uint32_t rounds = steps >= 2 ? 2 : 1;
    const uint64_t n_pad = (n + 127) / 128 * 128;
    const float b1 = 0.9f, b2 = 0.999f, lr = 0.02f;
    const size_t shm = train_smem_bytes(k, d);
    if (shm > 220 * 1024) return set_error(EJOIN_EUNSUPPORTED, "projection too large for training");
    auto step_fn = k <= 8 ? train_step_kernel<8> : train_step_kernel<16>;
    EJ_CUDA(cudaFuncSetAttribute(step_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
    const uint32_t tp = train_tile_pairs(d);
    unsigned sample_grid = 1;
    {
        int sms = 0, dev = 0;
        EJ_CUDA(cudaGetDevice(&dev));
        EJ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        sample_grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((M + 7) / 8, (uint64_t)sms * 8));
    }
    // a few blocks per SM, each accumulating its partial gradient in shared memory
    const unsigned grid = (unsigned)std::min<uint64_t>((B + tp - 1) / tp, 304);
    uint32_t t_step = 0;
    uint64_t cursor = 0;
    for (uint32_t r = 0; r < rounds; ++r) {
        DBuf<uint32_t> perm;
        EJ_TRY(learned_order(Y32, nullptr, bad, n, n_pad, d, P.p, k, 0.0f, lead_only, perm,
                             nullptr, s));
        sample_pairs_kernel<<<sample_grid, 256, 0, s>>>(
            Y32, bad, n, d, perm.p, M, seed + 7919ull * (r + 1), eps, 256, PairBatch{V.p, tgt.p});
        EJ_CUDA(cudaGetLastError());
        note_launch();
        const uint32_t nsteps = steps / rounds + (r < steps % rounds ? 1 : 0);
        for (uint32_t it = 0; it < nsteps; ++it, ++t_step) {
            if (cursor + B > M) cursor = 0;
            PairBatch pb{V.p + cursor * d, tgt.p + cursor};
            cursor += B;
            const float c1 = 1.0f - powf(b1, (float)(t_step + 1));
            const float c2 = 1.0f - powf(b2, (float)(t_step + 1));
            const AdamArgs ad{m1.p, m2.p, lr, b1, b2, c1, c2, done.p};
            step_fn<<<grid, TRAIN_THREADS, shm, s>>>(P.p, k, d, pb, B, ad, G.p, loss.p + t_step);
            EJ_CUDA(cudaGetLastError());
            note_launch();
        }
    }
    out.P.resize(nel);
    std::vector<unsigned long long> Lf(steps ? steps : 1);
    EJ_CUDA(cudaMemcpyAsync(out.P.data(), P.p, nel * sizeof(float), cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaMemcpyAsync(Lf.data(), loss.p, Lf.size() * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    std::vector<double> L(Lf.size());
    for (size_t i = 0; i < Lf.size(); ++i) L[i] = (double)(long long)Lf[i] / 1099511627776.0;
    // first / last loss averaged over a few steps (minibatch noise)
    const size_t w = std::min<size_t>(8, L.size());
    double a = 0, b = 0;
    for (size_t i = 0; i < w; ++i) {
        a += L[i];
        b += L[L.size() - 1 - i];
    }
    out.loss_first = a / w;
    out.loss_last = b / w;
    EJ_TRY(cert_spectral_norm(out.P.data(), k, d, &out.sigma_cert));
    return EJOIN_OK;
}

}  // namespace ejoin

// ------------------------------------------------------------ test hooks --

extern "C" int ejoin_testing_projection_grad(const float* V, const float* tgt, uint64_t M,
                                             const float* P, uint32_t k, uint32_t d, float* G_out,
                                             float* loss_out) {
    using namespace ejoin;
    clear_error();
    if (!V || !tgt || !P || !G_out || !loss_out || k == 0 || k > 16 || d == 0 || M == 0)
        return set_error(EJOIN_EINVAL, "bad arguments");
    cudaStream_t s = cudaStreamPerThread;
    DBuf<float> dV, dT, dP;
    DBuf<unsigned long long> dG, dL;
    EJ_TRY(dV.alloc(M * d, s, "V"));
    EJ_TRY(dT.alloc(M, s, "targets"));
    EJ_TRY(dP.alloc((size_t)k * d, s, "P"));
    EJ_TRY(dG.alloc((size_t)k * d, s, "G"));
    EJ_TRY(dL.alloc(1, s, "loss"));
    EJ_CUDA(cudaMemcpyAsync(dV.p, V, M * d * sizeof(float), cudaMemcpyHostToDevice, s));
    EJ_CUDA(cudaMemcpyAsync(dT.p, tgt, M * sizeof(float), cudaMemcpyHostToDevice, s));
    EJ_CUDA(cudaMemcpyAsync(dP.p, P, (size_t)k * d * sizeof(float), cudaMemcpyHostToDevice, s));
    EJ_TRY(dG.zero(s));
    EJ_TRY(dL.zero(s));
    const size_t shm = train_smem_bytes(k, d);
    auto fn = k <= 8 ? train_step_kernel<8> : train_step_kernel<16>;
    EJ_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
    PairBatch pb{dV.p, dT.p};
    fn<<<64, TRAIN_THREADS, shm, s>>>(dP.p, k, d, pb, M, AdamArgs{}, dG.p, dL.p);
    EJ_CUDA(cudaGetLastError());
    std::vector<unsigned long long> g((size_t)k * d);
    unsigned long long l = 0;
    EJ_CUDA(cudaMemcpyAsync(g.data(), dG.p, g.size() * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaMemcpyAsync(&l, dL.p, sizeof l, cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    for (size_t e = 0; e < g.size(); ++e) G_out[e] = (float)((double)(long long)g[e] / kFix);
    *loss_out = (float)((double)(long long)l / kFix);
    return EJOIN_OK;
}

extern "C" int ejoin_testing_renormalise(float* P, uint32_t k, uint32_t d, float* sigma_est_out) {
    using namespace ejoin;
    clear_error();
    if (!P || k == 0 || k > 16 || d == 0) return set_error(EJOIN_EINVAL, "bad arguments");
    cudaStream_t s = cudaStreamPerThread;
    DBuf<float> dP, dZ, dS;
    DBuf<unsigned long long> dG;
    const size_t nel = (size_t)k * d;
    EJ_TRY(dP.alloc(nel, s, "P"));
    EJ_TRY(dZ.alloc(2 * nel, s, "zero state"));
    EJ_TRY(dG.alloc(nel, s, "zero gradient"));
    EJ_TRY(dS.alloc(1, s, "sigma"));
    EJ_TRY(dZ.zero(s));
    EJ_TRY(dG.zero(s));
    EJ_CUDA(cudaMemcpyAsync(dP.p, P, nel * sizeof(float), cudaMemcpyHostToDevice, s));
    // zero gradient and learning rate: the Adam part leaves P unchanged
    const size_t ashm = nel * sizeof(float);
    if (ashm > 220 * 1024) return set_error(EJOIN_EUNSUPPORTED, "projection too large");
    EJ_CUDA(cudaFuncSetAttribute(adam_renorm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)ashm));
    adam_renorm_kernel<<<1, 256, ashm, s>>>(dP.p, dG.p, dZ.p, dZ.p + nel, k, d, 0.0f, 0.9f, 0.999f,
                                         1.0f, 1.0f, 1, dS.p);
    EJ_CUDA(cudaGetLastError());
    EJ_CUDA(cudaMemcpyAsync(P, dP.p, nel * sizeof(float), cudaMemcpyDeviceToHost, s));
    if (sigma_est_out)
        EJ_CUDA(cudaMemcpyAsync(sigma_est_out, dS.p, sizeof(float), cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    return EJOIN_OK;
}
