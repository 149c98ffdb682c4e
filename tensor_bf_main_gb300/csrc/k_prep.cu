// k_prep.cu -- centring, norms and operand packing for the Gram screens.
//
// Re-designs the reference's convertDataset (kernel_join.cu:44-54, a plain
// FP64 -> FP16 cast) and preComputedSquaredCoordinates (kernel_join.cu:57-88,
// partial squared norms per 16-wide chunk).  Here one pass per row:
//   y = fl(x - mu)       FP64 centring (mu = mean of the finite rows)
//   z = s * y            exact power-of-two scale
//   q = hi (+ lo)        operands in BF16/FP16 (hi + lo split) or FP8
// and, in FP64, the per-row quantities of the rigorous error bound: the
// norm of q, the quantisation residual ||z - q|| (exact per coordinate), the
// centring error, and from them the in-threshold alpha (carried by the GEMM
// itself in three extra K columns, see k_umma.cu) and the out-margin beta.
//
// Every stored operand is zero or a normal number of its format: values below
// the smallest normal are flushed here, so the tensor cores never see a
// subnormal input and the residual accounts for the flush exactly.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <string.h>

#include <algorithm>

#include "ejoin_internal.cuh"

namespace ejoin {
namespace {

// ------------------------------------------------------------- centring --
//
// mu is the FP32-representable mean of up to kMeanSample rows spread evenly
// over the data (finite values only).  Any fixed mu keeps every bound below
// rigorous; the mean only keeps the centred magnitudes small.
constexpr uint64_t kMeanSample = 65536;
constexpr uint32_t kMeanRowsPerBlock = 256;

__global__ void sample_colsum_kernel(const double* __restrict__ X, uint64_t n, uint32_t d,
                                     uint64_t S, double* psum, uint32_t* pcnt) {
    const uint64_t j0 = blockIdx.x * (uint64_t)kMeanRowsPerBlock;
    const uint64_t j1 = min(S, j0 + kMeanRowsPerBlock);
    for (uint32_t k = threadIdx.x; k < d; k += blockDim.x) {
        double s = 0.0;
        uint32_t c = 0;
#pragma unroll 8
        for (uint64_t j = j0; j < j1; ++j) {
            // j * n / S, evenly spread and increasing; S is n or the constant
            // kMeanSample, so no run-time 64-bit division (emulated on the GPU)
            const uint64_t row = S == n ? j : j * n / kMeanSample;
            const double v = X[row * d + k];
            if (isfinite(v)) {
                s += v;
                ++c;
            }
        }
        psum[blockIdx.x * (uint64_t)d + k] = s;
        pcnt[blockIdx.x * (uint64_t)d + k] = c;
    }
}

// mu_k = fl32(sum / count) in a fixed order (deterministic); 0 without data
// or beyond 1e30 (such data leaves the FP32 path anyway).
__global__ void sample_mean_kernel(const double* __restrict__ psum, const uint32_t* __restrict__ pcnt,
                                   uint32_t nb, uint32_t d, double* mu, float* muf) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d) return;
    double s = 0.0;
    uint64_t c = 0;
    for (uint32_t b = 0; b < nb; ++b) {
        s += psum[(uint64_t)b * d + k];
        c += pcnt[(uint64_t)b * d + k];
    }
    const double m = c ? s / (double)c : 0.0;
    const float f = fabs(m) < 1e30 ? (float)m : 0.0f;
    muf[k] = f;
    mu[k] = (double)f;
}

// a given FP32-representable mean (stored as double) as FP32
__global__ void mu_float_kernel(const double* __restrict__ mu, uint32_t d, float* muf) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < d) muf[k] = (float)mu[k];
}

constexpr uint32_t kCenterRange = 1u;  // a finite |x| >= 2^120: FP32 path unusable
constexpr uint32_t kCenterFlush = 2u;  // a nonzero |x| < 2^-126 was replaced by 0

struct CenterAcc {
    unsigned long long ngood;
    uint32_t maxy;  // bits of max |Y| (non-negative floats order like their bits)
    uint32_t flags;
};

// Y = fl32(x - mu) to within  |Y - (x - mu)| <= c_rel |Y| + e  (exact real
// x - mu, c_rel = 2^-23 (1 + 2^-23)), using integer and FP32 operations only
// (FP64 arithmetic is scarce on this GPU).  With E the biased exponent of x:
//  * 2^-126 <= |x| < 2^120: xf1 = x truncated to 24 significant bits (an FP32
//    normal, built from the bit fields), rem = x - xf1 = (low 29 mantissa
//    bits) * 2^(E-1075), |rem| < 2^-23 |x|.  If 2^(E-1075) is an FP32 normal
//    (E >= 949), xf2 = fl32(rem) (one rounding, the power-of-two product is
//    exact); otherwise xf2 = 0.  a = fl32(xf1 - mu), Y = fl32(a + xf2).
//    Round-to-nearest gives |Y - (a + xf2)| <= u|Y| + 2^-150,
//    |a - (xf1 - mu)| <= u|a|, |a| <= (1 + u)|Y| + 2^-150 + |xf2|, hence
//      xf2 kept:    e = 2^-46 (1 + 2^-20) |xf1| + 2^-148
//      xf2 dropped: e = |rem| <= 2^-23 (1 + 2^-22) |xf1|  (a = Y exactly)
//  * |x| < 2^-126: x is replaced by 0, Y = -mu exactly, e = 2^-126.
//  * |x| >= 2^120 (finite): flagged; the caller leaves the FP32 path.
__device__ __forceinline__ float center_coord(double x, float mu, float& e, uint32_t& flags,
                                              bool& finite) {
    const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
    const uint32_t E = (hi >> 20) & 0x7ffu;
    const uint32_t sgn = hi & 0x80000000u;
    finite = E != 0x7ffu;
    float xf1 = 0.0f, xf2 = 0.0f;
    e = 0.0f;
    if (E >= 897u && E <= 1142u) {
        xf1 = __uint_as_float(sgn | ((E - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
        if (E >= 949u) {
            xf2 = __fmul_rn(__uint2float_rn(lo & 0x1fffffffu), __uint_as_float((E - 948u) << 23));
            xf2 = __uint_as_float(__float_as_uint(xf2) | sgn);
            e = __fmaf_ru(fabsf(xf1), 1.4210854715202004e-14f * 1.00000095367431640625f,
                          3.5873240686715317e-43f);  // 2^-46 (1 + 2^-20), 2^-148
        } else {
            e = __fmul_ru(fabsf(xf1), 1.1920928955078125e-07f * 1.0000002384185791f);  // 2^-23 (1 + 2^-22)
        }
    } else if (E <= 896u) {
        if ((hi & 0x7fffffffu) | lo) {
            e = 1.1754943508222875e-38f;  // 2^-126
            flags |= kCenterFlush;
        }
    } else if (finite) {
        flags |= kCenterRange;
    }
    return __fadd_rn(__fsub_rn(xf1, mu), xf2);
}

// One pass over X: bad[i] (a non-finite coordinate), Y32 = the FP32 centred
// copy (0 for bad rows), Yerr[i] >= ||Y32_i - (x_i - mu)||_2 (rounded up:
// c_rel ||Y32_i|| + sum of the per-coordinate e), and the global maximum of
// |Y32| over good rows, their count and the range flags.  A warp handles
// ROWS rows per step with all loads issued first (VEC = 2: 16-byte loads of
// coordinate pairs, d even); without Y32 only bad and the count are written.
template <int VEC, int ROWS>
__global__ void __launch_bounds__(256) center_kernel(const double* __restrict__ X, uint64_t n,
                                                     uint32_t d, const float* __restrict__ muf,
                                                     uint8_t* __restrict__ bad,
                                                     float* __restrict__ Y32,
                                                     float* __restrict__ Yerr, CenterAcc* acc) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    const uint32_t nv = d / VEC;  // vectors per row
    float my = 0.0f;
    uint32_t fl = 0, ng = 0;
    for (uint64_t r0 = gw * ROWS; r0 < n; r0 += nw * ROWS) {
        bool fin[ROWS];
        float s2[ROWS], se[ROWS], rmax[ROWS];
        uint32_t rfl[ROWS];
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            fin[r] = true;
            s2[r] = se[r] = rmax[r] = 0.0f;
            rfl[r] = 0;
        }
        for (uint32_t v0 = 0; v0 < nv; v0 += 32) {
            const uint32_t v = v0 + lane;
            double xv[ROWS][VEC];
#pragma unroll
            for (int r = 0; r < ROWS; ++r) {
                const bool ok = r0 + r < n && v < nv;
                if (VEC == 2) {
                    const double2 t = ok ? reinterpret_cast<const double2*>(X + (r0 + r) * d)[v]
                                         : make_double2(0.0, 0.0);
                    xv[r][0] = t.x;
                    xv[r][VEC - 1] = t.y;
                } else {
                    xv[r][0] = ok ? X[(r0 + r) * d + v] : 0.0;
                }
            }
            if (v >= nv) continue;
#pragma unroll
            for (int r = 0; r < ROWS; ++r) {
                if (r0 + r >= n) continue;
                float y[VEC];
#pragma unroll
                for (int c = 0; c < VEC; ++c) {
                    float e;
                    bool f;
                    y[c] = center_coord(xv[r][c], muf[v * VEC + c], e, rfl[r], f);
                    fin[r] &= f;
                    s2[r] = __fmaf_ru(y[c], y[c], s2[r]);
                    se[r] = __fadd_ru(se[r], e);
                    rmax[r] = fmaxf(rmax[r], fabsf(y[c]));
                }
                if (Y32) {
                    float* yr = Y32 + (r0 + r) * d;
                    if (VEC == 2) reinterpret_cast<float2*>(yr)[v] = make_float2(y[0], y[VEC - 1]);
                    else yr[v] = y[0];
                }
            }
        }
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const uint64_t row = r0 + r;
            if (row >= n) continue;  // warp-uniform
            const bool good = __all_sync(0xffffffffu, fin[r]);
            float a = s2[r], b = se[r];
            for (int o = 16; o; o >>= 1) {
                a = __fadd_ru(a, __shfl_xor_sync(0xffffffffu, a, o));
                b = __fadd_ru(b, __shfl_xor_sync(0xffffffffu, b, o));
            }
            if (good) {
                my = fmaxf(my, rmax[r]);
                fl |= rfl[r];
                ng += lane == 0;
            } else if (Y32) {
                for (uint32_t k = lane; k < d; k += 32) Y32[row * d + k] = 0.0f;
            }
            if (lane == 0) {
                bad[row] = good ? 0 : 1;
                if (Yerr)
                    Yerr[row] = good ? __fmaf_ru(1.1920930376163766e-07f, __fsqrt_ru(a), b) : 0.0f;
            }
        }
    }
    // block-level merge, one set of atomics per block
    for (int o = 16; o; o >>= 1) {
        my = fmaxf(my, __shfl_xor_sync(0xffffffffu, my, o));
        fl |= __shfl_xor_sync(0xffffffffu, fl, o);
        ng += __shfl_xor_sync(0xffffffffu, ng, o);
    }
    __shared__ float smy[8];
    __shared__ uint32_t sfl[8], sng[8];
    const uint32_t w = threadIdx.x / 32;
    if (lane == 0) {
        smy[w] = my;
        sfl[w] = fl;
        sng[w] = ng;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (uint32_t i = 1; i < blockDim.x / 32; ++i) {
            my = fmaxf(my, smy[i]);
            fl |= sfl[i];
            ng += sng[i];
        }
        if (ng) atomicAdd(&acc->ngood, (unsigned long long)ng);
        if (my > 0.0f) atomicMax(&acc->maxy, __float_as_uint(my));
        if (fl) atomicOr(&acc->flags, fl);
    }
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------ format rounding --

struct FmtInfo {
    int fbits;          // fraction bits
    double min_normal;  // smallest positive normal
};
__device__ __forceinline__ FmtInfo fmt_info(Fmt f) {
    if (f == Fmt::BF16) return {7, 1.1754943508222875e-38};  // 2^-126
    if (f == Fmt::FP16) return {10, 6.103515625e-05};        // 2^-14
    return {3, 0.015625};                                     // E4M3: 2^-6
}

// Round v to `fbits` fraction bits (ties to even) and flush results below the
// format's smallest normal to zero.  v is a normal double (or zero).
__device__ __forceinline__ double round_fmt(double v, FmtInfo fi) {
    if (fabs(v) < fi.min_normal) return 0.0;
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int sh = 52 - fi.fbits;
    unsigned long long lsb = (b >> sh) & 1ull;
    b += ((1ull << (sh - 1)) - 1ull) + lsb;
    b &= ~((1ull << sh) - 1ull);
    double r = __longlong_as_double((long long)b);
    return fabs(r) < fi.min_normal ? 0.0 : r;
}

// Smallest representable value of the format >= v (normal or zero).
__device__ __forceinline__ double round_fmt_up(double v, FmtInfo fi) {
    double r = round_fmt(v, fi);
    if (r >= v) return r;
    if (r == 0.0) return v > 0.0 ? fi.min_normal : 0.0;  // v in (-min_normal, 0): 0 >= v
    int e;
    frexp(fabs(r), &e);  // |r| in [2^(e-1), 2^e)
    double ulp = ldexp(1.0, e - 1 - fi.fbits);
    double up = r + ulp;  // exact; crossing towards zero stays representable
    return fabs(up) < fi.min_normal ? 0.0 : up;
}

__device__ __forceinline__ uint16_t to_bits16(double r, Fmt f) {
    float x = (float)r;  // exact: r already has <= 11 significant bits
    if (f == Fmt::BF16) return (uint16_t)(__float_as_uint(x) >> 16);
    return __half_as_ushort(__float2half_rn(x));
}

// ------------------------------------------------------------ DMMA pack --

__global__ void pack_dmma_kernel(const double* __restrict__ X, uint64_t n, uint64_t n_pad,
                                 const uint32_t* __restrict__ perm, const uint8_t* __restrict__ bad,
                                 const double* __restrict__ mu, DmmaParams P, double* Y, double* h,
                                 double* g) {
    const uint64_t p = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (p >= n_pad) return;
    const uint64_t src = p < n ? (perm ? perm[p] : p) : 0;
    const bool good = p < n && !bad[src];
    double nrm = 0.0;
    for (uint32_t k = lane; k < P.dp; k += 32) {
        double y = 0.0;
        if (good && k < P.d) y = __dsub_rn(X[src * P.d + k], mu[k]);
        Y[p * P.dp + k] = y;
        nrm = __fma_rn(y, y, nrm);
    }
    nrm = warp_sum(nrm);
    if (lane) return;
    if (!good) {
        h[p] = INFINITY;
        g[p] = INFINITY;
        return;
    }
    const double gs = (P.d + 4) * kU;
    // FP64 underflow: every square, product and rounded sum may lose up to
    // 2^-1074 in absolute terms (relevant for data near the bottom of the
    // double range); these absolute terms join the relative bounds below
    const double tiny = (2.0 * P.dp + P.d + 16) * 4.9406564584124654e-324;
    const double nup = nrm * (1 + gs) + tiny, ndn = nrm * (1 - gs) - tiny;
    const double rho = 1.0001 * kU * sqrt(nup) * (1 + 8 * kU) + tiny;
    // in:  G >= h_i + h_j   (h rounded up, incl. epilogue subtraction rounding)
    double hv = 0.5 * (nup * (1 + P.crel) + 2.0 * P.sTlo * rho - 0.5 * P.Tlo) + tiny;
    hv += 8 * kU * (nup + fabs(hv) + P.Tlo + P.sTlo * rho);
    // out: G <  g_i + g_j   (g rounded down)
    double gv = 0.5 * (ndn - P.crel * nup - 0.5 * P.Thi - 2.0 * P.sThi * rho - 2.0 * rho * rho) - tiny;
    gv -= 8 * kU * (nup + fabs(gv) + P.Thi + P.sThi * rho);
    h[p] = hv;
    g[p] = gv;
}

// --------------------------------------------------- 16-bit screen pack --

// Round a float to `fbits` fraction bits (ties to even); results below the
// format's smallest normal are flushed to zero.
__device__ __forceinline__ float round_fmt_f(float v, int fbits, float min_normal) {
    if (fabsf(v) < min_normal) return 0.0f;
    uint32_t b = __float_as_uint(v);
    const int sh = 23 - fbits;
    const uint32_t lsb = (b >> sh) & 1u;
    b += ((1u << (sh - 1)) - 1u) + lsb;
    b &= ~((1u << sh) - 1u);
    const float r = __uint_as_float(b);
    return fabsf(r) < min_normal ? 0.0f : r;
}

// Squared norm of q accumulated in FP32 (round to nearest): each term passes
// through at most `chain` lane-chain FMAs and `levels` shuffle-tree additions,
// so |computed - exact| <= gamma * exact + (dp + 160) 2^-149 (underflow), with
// gamma = (chain + levels + 1) 2^-24 (1.01 covers gamma_m's denominator).
struct NormBound {
    double rel, abs;
};
__device__ __forceinline__ NormBound fp32_norm_bound(uint32_t dp, uint32_t chain, uint32_t levels) {
    return {(chain + levels + 1) * 5.9604644775390625e-08 * 1.01, (dp + 160) * 1.4012984643248171e-45};
}

// Bit pattern of a value already representable in the 16-bit format.
__device__ __forceinline__ uint16_t bits16f(float x, Fmt f) {
    if (f == Fmt::BF16) return (uint16_t)(__float_as_uint(x) >> 16);
    return __half_as_ushort(__float2half_rn(x));
}

// A warp packs 32 consecutive rows.  Phase 1, two rows at a time (half-warp
// h takes row 2 it + h; lane l of the half handles coordinates 4l .. 4l+3 of
// every 64-wide slab, 16-byte loads): z = s * Y32 (exact power-of-two scaling
// of the FP32 centred copy), hi = round(z), lo = round(z - hi) (split),
// ef = z - hi - lo; every FP32 subtraction here is exact.  The residual to the
// exact centred point is (Yerr_i s, from the centring pass) + |ef| (+ 2^-126
// per flushed coordinate).  Per row: nq = |q|^2 (FP32, bounded by
// fp32_norm_bound) and in FP32 rounded up: |ef|^2, |(|hi| + |lo|)|^2, |lo|^2.
// The FP32 coordinates z and a per-row radius go to Xf / rad for the FP32
// band pre-check.  Phase 2 (lane L = row 2 (L % 16) + L / 16, whose sums the
// half-warp reduction left in that lane): the FP64 threshold arithmetic
// (alpha, beta), the aug slab.
template <Fmt F>
__global__ void __launch_bounds__(256) pack16_kernel(const float* __restrict__ Y32, uint64_t n,
                                                     uint64_t n_pad,
                                                     const uint32_t* __restrict__ perm,
                                                     const uint8_t* __restrict__ bad,
                                                     const float* __restrict__ Yerr, ScreenParams P,
                                                     uint16_t* Q, uint16_t* Aug, float* beta,
                                                     float* Xf, float* rad) {
    const uint64_t p0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32 * 32;
    const uint32_t lane = threadIdx.x & 31, hw = lane >> 4, l = lane & 15;
    if (p0 >= n_pad) return;
    const FmtInfo fi = fmt_info(F);
    const float mnf = (float)fi.min_normal;
    const float sf = (float)P.scale;
    // 16-byte access to Y32 / Xf rows needs d % 4 == 0 (and aligned bases)
    const bool v4 = P.d % 4 == 0 && (((uintptr_t)Y32 | (uintptr_t)Xf) & 15) == 0;
    float m_nq = 0, m_e2 = 0, m_a2 = 0, m_l2 = 0;
    uint64_t m_src = 0;
    bool m_good = false;
    // the warp's 32 source rows and their flags, loaded once (lane r: row
    // p0 + r) and handed out by shuffles, so that no index load sits in
    // front of each row's gather
    const uint64_t pl = p0 + lane;
    const uint64_t src_l = pl < n ? (perm ? perm[pl] : pl) : 0;
    const uint32_t good_l = (pl < n && !bad[src_l]) ? 1u : 0u;
    for (uint32_t it = 0; it < 16; ++it) {
        const uint64_t p = p0 + 2 * it + hw;
        const uint64_t src = __shfl_sync(0xffffffffu, src_l, 2 * it + hw);
        const bool good = __shfl_sync(0xffffffffu, good_l, 2 * it + hw) != 0u;
        uint16_t* row = Q + p * (uint64_t)P.width;
        float nq = 0, e2 = 0, a2 = 0, l2 = 0;
        for (uint32_t k0 = 4 * l; k0 < P.dp; k0 += 64) {
            float z[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (good && k0 < P.d) {
                if (v4) {
                    const float4 y = __ldg(reinterpret_cast<const float4*>(Y32 + src * P.d + k0));
                    z[0] = y.x;
                    z[1] = y.y;
                    z[2] = y.z;
                    z[3] = y.w;
                } else {
#pragma unroll
                    for (int t = 0; t < 4; ++t)
                        if (k0 + t < P.d) z[t] = __ldg(&Y32[src * P.d + k0 + t]);
                }
            }
            uint16_t hb[4], lb[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                float zf = z[t] * sf;  // exact power-of-two scaling
                if (fabsf(zf) < 1.1754944e-38f) zf = 0.0f;  // keep Xf free of FP32 subnormals
                const float hi = round_fmt_f(zf, fi.fbits, mnf);
                float ef = zf - hi;  // exact
                float lo = 0.0f;
                if (P.split) {
                    lo = round_fmt_f(ef, fi.fbits, mnf);
                    ef = ef - lo;  // exact
                }
                const float q = hi + lo;  // exact
                nq = __fmaf_rn(q, q, nq);
                const float aq = fabsf(hi) + fabsf(lo);  // exact
                e2 = __fmaf_ru(ef, ef, e2);
                a2 = __fmaf_ru(aq, aq, a2);
                l2 = __fmaf_ru(lo, lo, l2);
                hb[t] = bits16f(hi, F);
                lb[t] = bits16f(lo, F);
                z[t] = zf;
            }
            // k0 is a multiple of 4 and rows are 128-byte multiples: 8-byte stores
            *reinterpret_cast<uint2*>(row + k0) =
                make_uint2(hb[0] | ((uint32_t)hb[1] << 16), hb[2] | ((uint32_t)hb[3] << 16));
            if (P.split)
                *reinterpret_cast<uint2*>(row + P.dp + k0) =
                    make_uint2(lb[0] | ((uint32_t)lb[1] << 16), lb[2] | ((uint32_t)lb[3] << 16));
            if (k0 < P.d) {
                if (v4) {
                    *reinterpret_cast<float4*>(Xf + p * P.d + k0) = make_float4(z[0], z[1], z[2], z[3]);
                } else {
#pragma unroll
                    for (int t = 0; t < 4; ++t)
                        if (k0 + t < P.d) Xf[p * P.d + k0 + t] = z[t];
                }
            }
        }
        // reduction within the half-warp (xor offsets < 16 stay in the half)
        for (int o = 8; o; o >>= 1) {
            nq = __fadd_rn(nq, __shfl_xor_sync(0xffffffffu, nq, o));
            e2 = __fadd_ru(e2, __shfl_xor_sync(0xffffffffu, e2, o));
            a2 = __fadd_ru(a2, __shfl_xor_sync(0xffffffffu, a2, o));
            l2 = __fadd_ru(l2, __shfl_xor_sync(0xffffffffu, l2, o));
        }
        if (l == it) {
            m_nq = nq;
            m_e2 = e2;
            m_a2 = a2;
            m_l2 = l2;
            m_src = src;
            m_good = good;
        }
    }
    // ---- phase 2: row p0 + 2 (lane % 16) + lane / 16
    const uint64_t p = p0 + 2 * l + hw;
    double ah[3] = {0, 0, 0};
    double b = 0.0;
    float radius = INFINITY;  // bad and padding rows: the FP32 pre-check never decides
    if (m_good) {
        const NormBound nb = fp32_norm_bound(P.dp, P.dp / 16, 4);
        const double nup = (double)m_nq * (1 + nb.rel) + nb.abs;
        const double ndn = (double)m_nq * (1 - nb.rel) - nb.abs;
        const double a2u = (double)m_a2, lu = (double)m_l2;
        // distance of the FP32 coordinates from the exact scaled centred point:
        // the centring bound (exact scaling) plus values flushed below 2^-126
        const double zerr = ((double)__ldg(&Yerr[m_src]) * P.scale +
                             P.flush_err) * (1 + 4 * kU);
        // FP32 square root rounded up: an upper bound, without an FP64 square
        // root (FP64 runs at a small fraction of FP32 on GB300)
        const double rho = ((double)__fsqrt_ru(m_e2) * (1 + 1e-7) + zerr) * (1 + 8 * kU);
        radius = __double2float_ru(zerr);
        const double m2 = acc_margin2(P, a2u, lu);
        double R = nup + m2 + lu + P.absacc - 0.5 * P.Tlo + 2.0 * P.sTlo * rho;
        R += 12 * kU * (nup + m2 + lu + P.absacc + 0.5 * P.Tlo + 2.0 * P.sTlo * rho);
        // R / (2 (1 -/+ cacc_al)) as a product with reciprocals rounded towards
        // a larger alpha on the host; the margin below covers the product's
        // rounding
        double at = R * (R >= 0 ? P.inv_in_pos : P.inv_in_neg);
        at += fabs(at) * 4 * kU;
        at = fmax(at, P.clamp_lo);
        ah[0] = round_fmt(at, fi);
        const double r1 = __dsub_rn(at, ah[0]);
        ah[1] = round_fmt(r1, fi);
        const double r2 = __dsub_rn(r1, ah[1]);
        ah[2] = round_fmt_up(r2, fi);
        const double alpha = ah[0] + ah[1] + ah[2];  // >= at (ah[2] >= r2)
        b = 0.5 * P.Thi + 2.0 * P.sThi * rho + 2.0 * rho * rho - ndn + 2.0 * alpha +
            m2 + 2.0 * P.cacc_al * fabs(alpha) + lu + P.absacc;
        b += 12 * kU * (0.5 * P.Thi + 2.0 * P.sThi * rho + 2.0 * rho * rho + ndn + 2.0 * fabs(alpha) +
                        m2 + 2.0 * P.cacc_al * fabs(alpha) + lu + P.absacc);
        b *= 0.5;
    } else {
        // never in, never band: C = q_i.q_j - alpha_i - alpha_j << -W
        ah[0] = (F == Fmt::FP16) ? 32768.0 : kTwo100;
    }
    // aug row: A side [a0 a1 a2 -1 -1 -1 0 ..] (16), B side [-1 -1 -1 a0 a1 a2 0 ..] (16)
    uint16_t vals[32];
#pragma unroll
    for (int e = 0; e < 32; ++e) vals[e] = 0;
    const uint16_t m1 = to_bits16(-1.0, F);
    vals[0] = to_bits16(ah[0], F);
    vals[1] = to_bits16(ah[1], F);
    vals[2] = to_bits16(ah[2], F);
    vals[3] = vals[4] = vals[5] = m1;
    vals[16] = vals[17] = vals[18] = m1;
    vals[19] = vals[0];
    vals[20] = vals[1];
    vals[21] = vals[2];
    uint4* aug = reinterpret_cast<uint4*>(Aug + p * 32);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        uint4 w;
        w.x = vals[8 * v + 0] | ((uint32_t)vals[8 * v + 1] << 16);
        w.y = vals[8 * v + 2] | ((uint32_t)vals[8 * v + 3] << 16);
        w.z = vals[8 * v + 4] | ((uint32_t)vals[8 * v + 5] << 16);
        w.w = vals[8 * v + 6] | ((uint32_t)vals[8 * v + 7] << 16);
        aug[v] = w;
    }
    beta[p] = m_good ? __double2float_ru(b) : 0.0f;
    rad[p] = radius;
}

// ----------------------------------------------------------- FP8 pack --

// E4M3 operands with a per-row power-of-two scale sigma_i (|z / sigma| <= 240,
// below the format's 448 limit).  A warp packs 32 rows; per row the lanes keep
// their FP32 coordinates zf in registers (d <= 1024), take the row maximum,
// then quantise f = round_e4m3(zf / sigma) (division by a power of two is
// exact), q = sigma f, residual zf - q exact in FP32.  Phase 2 (lane = row):
// alpha in Gram units as for the 16-bit screen, stored for the BF16 aug MMA
// as  A = [alpha/sigma (3 BF16 terms, last rounded up), 1/sigma x3],
//     B = [-1/sigma x3, -alpha/sigma (3 terms)],
// so that the accumulator, in units of F = f_i . f_j, holds
// F - (alpha_i + alpha_j) / (sigma_i sigma_j).
constexpr int PACK8_MAXV = 32;  // coordinates per lane: d <= 1024
__global__ void __launch_bounds__(256) pack8_kernel(const float* __restrict__ Y32, uint64_t n,
                                                    uint64_t n_pad,
                                                    const uint32_t* __restrict__ perm,
                                                    const uint8_t* __restrict__ bad,
                                                    const float* __restrict__ Yerr, ScreenParams P,
                                                    uint8_t* Q, uint16_t* Aug, float* beta,
                                                    float* sig, float* Xf, float* rad,
                                                    uint16_t* Xh, float* radh) {
    const uint64_t p0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32 * 32;
    const uint32_t lane = threadIdx.x & 31;
    if (p0 >= n_pad) return;
    const float mnf = 0.015625f;  // E4M3 smallest normal 2^-6
    float m_nq = 0, m_e2 = 0, m_eh = 0, m_sig = 1.0f;
    uint64_t m_src = 0;
    bool m_good = false;
    // the warp's 32 source rows and their flags, loaded once and shuffled
    const uint64_t pl = p0 + lane;
    const uint64_t src_l = pl < n ? (perm ? perm[pl] : pl) : 0;
    const uint32_t good_l = (pl < n && !bad[src_l]) ? 1u : 0u;
    for (uint32_t r = 0; r < 32; ++r) {
        const uint64_t p = p0 + r;
        const uint64_t src = __shfl_sync(0xffffffffu, src_l, r);
        const bool good = __shfl_sync(0xffffffffu, good_l, r) != 0u;
        float zv[PACK8_MAXV];
        float mx = 0.0f;
#pragma unroll
        for (int t = 0; t < PACK8_MAXV; ++t) {
            const uint32_t k = lane + 32u * t;
            float zf = 0.0f;
            if (good && k < P.d) {
                zf = Y32[src * P.d + k] * (float)P.scale;  // exact power-of-two scaling
                if (fabsf(zf) < 1.1754944e-38f) zf = 0.0f;
            }
            zv[t] = zf;
            mx = fmaxf(mx, fabsf(zf));
        }
        for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        // sigma = 2^ceil(log2(mx / 240)), 1 for an all-zero row
        float sgm = 1.0f;
        if (mx > 0.0f) {
            int e;
            frexpf(mx / 240.0f, &e);  // mx/240 in [2^(e-1), 2^e)
            sgm = ldexpf(1.0f, e);
        }
        const float inv = 1.0f / sgm;  // exact (power of two)
        float nq = 0, e2 = 0, eh = 0;
        uint8_t* row = Q + p * (uint64_t)P.width;
#pragma unroll
        for (int t = 0; t < PACK8_MAXV; ++t) {
            const uint32_t k = lane + 32u * t;
            if (k >= P.dp) break;
            const float zf = zv[t];
            const float f = round_fmt_f(zf * inv, 3, mnf);
            const float q = f * sgm;        // exact
            const float ef = zf - q;        // exact
            nq = __fmaf_rn(q, q, nq);
            e2 = __fmaf_ru(ef, ef, e2);
            row[k] = (uint8_t)__nv_cvt_float_to_fp8(f, __NV_SATFINITE, __NV_E4M3);
            if (k < P.d) {
                Xf[p * P.d + k] = zf;
                if (Xh) {
                    // |zf| <= 1 (the scale): no overflow; zf - zh is exact
                    const __half hv = __float2half_rn(zf);
                    const float dh = zf - __half2float(hv);
                    eh = __fmaf_ru(dh, dh, eh);
                    Xh[p * P.d + k] = __half_as_ushort(hv);
                }
            }
        }
        for (int o = 16; o; o >>= 1) {
            nq = __fadd_rn(nq, __shfl_xor_sync(0xffffffffu, nq, o));
            e2 = __fadd_ru(e2, __shfl_xor_sync(0xffffffffu, e2, o));
            eh = __fadd_ru(eh, __shfl_xor_sync(0xffffffffu, eh, o));
        }
        if (lane == r) {
            m_nq = nq;
            m_e2 = e2;
            m_eh = eh;
            m_src = src;
            m_sig = sgm;
            m_good = good;
        }
    }
    // ---- phase 2: row p0 + lane
    const uint64_t p = p0 + lane;
    const FmtInfo bf = fmt_info(Fmt::BF16);
    double ah[3] = {0, 0, 0};
    double b = 0.0, rsig = 1.0;
    float radius = INFINITY;
    if (m_good) {
        const NormBound nb = fp32_norm_bound(P.dp, (P.dp + 31) / 32, 5);
        const double nup = (double)m_nq * (1 + nb.rel) + nb.abs;
        const double ndn = (double)m_nq * (1 - nb.rel) - nb.abs;
        const double a2u = nup;  // |(|q|)|^2 = |q|^2
        const double zerr = ((double)__ldg(&Yerr[m_src]) * P.scale +
                             P.flush_err) * (1 + 4 * kU);
        // FP32 square root rounded up: an upper bound, without an FP64 square
        // root (FP64 runs at a small fraction of FP32 on GB300)
        const double rho = ((double)__fsqrt_ru(m_e2) * (1 + 1e-7) + zerr) * (1 + 8 * kU);
        radius = __double2float_ru(zerr);
        const double m2 = acc_margin2(P, a2u, 0.0);
        double R = nup + m2 + P.absacc - 0.5 * P.Tlo + 2.0 * P.sTlo * rho;
        R += 12 * kU * (nup + m2 + P.absacc + 0.5 * P.Tlo + 2.0 * P.sTlo * rho);
        // R / (2 (1 -/+ cacc_al)) as a product with reciprocals rounded towards
        // a larger alpha on the host; the margin below covers the product's
        // rounding
        double at = R * (R >= 0 ? P.inv_in_pos : P.inv_in_neg);
        at += fabs(at) * 4 * kU;
        rsig = 1.0 / (double)m_sig;  // exact
        double as = fmax(at * rsig, -kTwo100);  // alpha / sigma, clamped upwards (safe)
        ah[0] = round_fmt(as, bf);
        const double r1 = __dsub_rn(as, ah[0]);
        ah[1] = round_fmt(r1, bf);
        const double r2 = __dsub_rn(r1, ah[1]);
        ah[2] = round_fmt_up(r2, bf);
        const double alpha = (ah[0] + ah[1] + ah[2]) * (double)m_sig;  // >= at
        b = 0.5 * P.Thi + 2.0 * P.sThi * rho + 2.0 * rho * rho - ndn + 2.0 * alpha +
            m2 + 2.0 * P.cacc_al * fabs(alpha) + P.absacc;
        b += 12 * kU * (0.5 * P.Thi + 2.0 * P.sThi * rho + 2.0 * rho * rho + ndn + 2.0 * fabs(alpha) +
                        m2 + 2.0 * P.cacc_al * fabs(alpha) + P.absacc);
        b *= 0.5;
    } else {
        ah[0] = kTwo100;  // never in, never band
        m_sig = 1.0f;
        rsig = 1.0;
    }
    uint16_t vals[32];
#pragma unroll
    for (int e = 0; e < 32; ++e) vals[e] = 0;
    const uint16_t rp = to_bits16(rsig, Fmt::BF16), rm = to_bits16(-rsig, Fmt::BF16);
    vals[0] = to_bits16(ah[0], Fmt::BF16);
    vals[1] = to_bits16(ah[1], Fmt::BF16);
    vals[2] = to_bits16(ah[2], Fmt::BF16);
    vals[3] = vals[4] = vals[5] = rp;
    vals[16] = vals[17] = vals[18] = rm;
    vals[19] = to_bits16(-ah[0], Fmt::BF16);
    vals[20] = to_bits16(-ah[1], Fmt::BF16);
    vals[21] = to_bits16(-ah[2], Fmt::BF16);
    uint4* aug = reinterpret_cast<uint4*>(Aug + p * 32);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        uint4 w;
        w.x = vals[8 * v + 0] | ((uint32_t)vals[8 * v + 1] << 16);
        w.y = vals[8 * v + 2] | ((uint32_t)vals[8 * v + 3] << 16);
        w.z = vals[8 * v + 4] | ((uint32_t)vals[8 * v + 5] << 16);
        w.w = vals[8 * v + 6] | ((uint32_t)vals[8 * v + 7] << 16);
        aug[v] = w;
    }
    beta[p] = m_good ? __double2float_ru(b) : 0.0f;
    sig[p] = m_good ? m_sig : INFINITY;  // padding / bad rows do not lower a tile's minimum
    rad[p] = radius;
    // radius of the FP16 copy: |zh - z| <= |zh - zf| + |zf - z| (rounded up)
    if (radh) radh[p] = __fadd_ru(radius, __fsqrt_ru(m_eh));
}

// per 128-row tile: min sigma of its rows (1 for a tile without finite rows)
__global__ void tile_min_sigma_kernel(const float* __restrict__ sig, uint64_t ntiles, float* tmin) {
    const uint64_t t = blockIdx.x;
    if (t >= ntiles) return;
    float m = INFINITY;
    for (int r = threadIdx.x; r < 128; r += blockDim.x) m = fminf(m, sig[t * 128 + r]);
    for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float sm[4];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x / 32] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = sm[0];
        for (int w = 1; w < (int)(blockDim.x / 32); ++w) r = fminf(r, sm[w]);
        tmin[t] = isinf(r) ? 1.0f : r;
    }
}

// Maximum of beta over every group of 32 consecutive rows (the column chunks
// of the Gram epilogue): a thread per row, one warp per group.
__global__ void chunk_max_kernel(const float* __restrict__ beta, uint64_t n_pad, float* cmax) {
    const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    float m = r < n_pad ? beta[r] : 0.0f;  // pad / bad rows carry 0
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && r < n_pad) cmax[r / 32] = m;
}

}  // namespace

int launch_center_stats(const double* X, uint64_t n, uint32_t d, uint8_t* bad, double* mu,
                        float* Y32, float* Yerr, CenterStats* out, cudaStream_t s, bool mu_given,
                        const StageCopy* sc, uint64_t prefix_rows, const PrefixHook* on_prefix) {
    *out = CenterStats{};
    DBuf<float> muf;
    EJ_TRY(muf.alloc(d, s, "FP32 mean"));
    const uint64_t S = std::min<uint64_t>(n, kMeanSample);
    const uint32_t nb = (uint32_t)((S + kMeanRowsPerBlock - 1) / kMeanRowsPerBlock);
    if (mu_given) {
        mu_float_kernel<<<(d + 127) / 128, 128, 0, s>>>(mu, d, muf.p);
        EJ_CUDA(cudaGetLastError());
        note_launch();
    } else if (nb) {
        DBuf<double> psum;
        DBuf<uint32_t> pcnt;
        EJ_TRY(psum.alloc((size_t)nb * d, s, "sample column sums"));
        EJ_TRY(pcnt.alloc((size_t)nb * d, s, "sample column counts"));
        // with a pending copy the sample rows are read from host memory
        sample_colsum_kernel<<<nb, 128, 0, s>>>(sc ? sc->host_dev : X, n, d, S, psum.p, pcnt.p);
        EJ_CUDA(cudaGetLastError());
        sample_mean_kernel<<<(d + 127) / 128, 128, 0, s>>>(psum.p, pcnt.p, nb, d, mu, muf.p);
        EJ_CUDA(cudaGetLastError());
        note_launch(2);
    } else {
        EJ_TRY(muf.zero(s));
        EJ_CUDA(cudaMemsetAsync(mu, 0, d * sizeof(double), s));
    }
    DBuf<CenterAcc> acc;
    EJ_TRY(acc.alloc(1, s, "centring totals"));
    EJ_TRY(acc.zero(s));
    if (n) {
        int sms = 0, dev = 0;
        EJ_CUDA(cudaGetDevice(&dev));
        EJ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        // one wave of resident blocks (8 warps, 4 rows per warp step)
        const bool vec = (d % 2 == 0) && (((uintptr_t)X & 15) == 0);
        auto fn = vec ? center_kernel<2, 4> : center_kernel<1, 4>;
        int per_sm = 0;
        EJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0));
        auto center = [&](uint64_t r0, uint64_t rows) -> int {
            const uint64_t want = (rows + 31) / 32;
            const unsigned grid = (unsigned)std::max<uint64_t>(
                1, std::min<uint64_t>(want, (uint64_t)sms * std::max(per_sm, 1)));
            fn<<<grid, 256, 0, s>>>(X + r0 * d, rows, d, muf.p, bad + r0,
                                    Y32 ? Y32 + r0 * d : nullptr, Yerr ? Yerr + r0 : nullptr,
                                    acc.p);
            EJ_CUDA(cudaGetLastError());
            note_launch();
            return EJOIN_OK;
        };
        // event on s after the centring of the first prefix_rows rows, handed
        // to on_prefix once every chunk is enqueued
        cudaEvent_t pev = nullptr;
        if (on_prefix) EJ_CUDA(cudaEventCreateWithFlags(&pev, cudaEventDisableTiming));
        struct EventGuard {
            cudaEvent_t& e;
            ~EventGuard() {
                if (e) cudaEventDestroy(e);
            }
        } pev_guard{pev};
        bool pev_recorded = false;
        auto mark_prefix = [&](uint64_t rows_done) -> int {
            if (pev && !pev_recorded && rows_done >= std::min(prefix_rows, n)) {
                EJ_CUDA(cudaEventRecord(pev, s));
                pev_recorded = true;
            }
            return EJOIN_OK;
        };
        if (!sc) {
            EJ_TRY(center(0, n));
            EJ_TRY(mark_prefix(n));
        } else {
            // chunked copy on a side stream; s waits for each chunk, then
            // centres it.  The side stream first waits for s (X was allocated
            // on s).  Chunk starts stay 16-byte aligned (even row counts).
            constexpr int kChunks = 8;
            cudaStream_t cs = nullptr;
            cudaEvent_t ev[kChunks + 1] = {};
            int rc = EJOIN_OK;
            auto fail = [&](cudaError_t e, const char* what) {
                if (rc == EJOIN_OK) rc = cuda_error(e, what, __FILE__, __LINE__);
            };
            cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
            if (e != cudaSuccess) fail(e, "cudaStreamCreateWithFlags");
            for (int c = 0; c <= kChunks && rc == EJOIN_OK; ++c) {
                e = cudaEventCreateWithFlags(&ev[c], cudaEventDisableTiming);
                if (e != cudaSuccess) fail(e, "cudaEventCreateWithFlags");
            }
            if (rc == EJOIN_OK) {
                if ((e = cudaEventRecord(ev[kChunks], s)) != cudaSuccess) fail(e, "cudaEventRecord");
                else if ((e = cudaStreamWaitEvent(cs, ev[kChunks], 0)) != cudaSuccess)
                    fail(e, "cudaStreamWaitEvent");
            }
            const uint64_t step = ((n + kChunks - 1) / kChunks + 1) & ~1ull;
            for (uint64_t r0 = 0, c = 0; r0 < n && rc == EJOIN_OK; r0 += step, ++c) {
                const uint64_t rows = std::min<uint64_t>(step, n - r0);
                e = cudaMemcpyAsync(const_cast<double*>(X) + r0 * d, sc->host + r0 * d,
                                    rows * d * sizeof(double), cudaMemcpyHostToDevice, cs);
                if (e != cudaSuccess) { fail(e, "cudaMemcpyAsync (points)"); break; }
                if ((e = cudaEventRecord(ev[c], cs)) != cudaSuccess) { fail(e, "cudaEventRecord"); break; }
                if ((e = cudaStreamWaitEvent(s, ev[c], 0)) != cudaSuccess) {
                    fail(e, "cudaStreamWaitEvent");
                    break;
                }
                rc = center(r0, rows);
                if (rc == EJOIN_OK) rc = mark_prefix(r0 + rows);
            }
            // on success s is ordered after every chunk copy; on failure no copy
            // may stay in flight into memory the caller frees.  The stream and
            // events are released once their work completes.
            if (rc != EJOIN_OK && cs) cudaStreamSynchronize(cs);
            for (int c = 0; c <= kChunks; ++c)
                if (ev[c]) cudaEventDestroy(ev[c]);
            if (cs) cudaStreamDestroy(cs);
            if (rc != EJOIN_OK) return rc;
        }
        // every copy and centring pass is enqueued: the prefix hook (projection
        // training on the first rows) runs while the rest still streams in
        if (pev_recorded) {
            const int hrc = (*on_prefix)(pev);
            if (hrc != EJOIN_OK) {
                cudaStreamSynchronize(s);
                return hrc;
            }
        }
    }
    CenterAcc h;
    EJ_CUDA(cudaMemcpyAsync(&h, acc.p, sizeof h, cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    float my;
    memcpy(&my, &h.maxy, sizeof my);
    out->maxy = (double)my;
    out->ngood = h.ngood;
    out->range = (h.flags & kCenterRange) != 0;
    out->flushed = (h.flags & kCenterFlush) != 0;
    return EJOIN_OK;
}

int launch_pack_dmma(const double* X, uint64_t n, uint64_t n_pad, const uint32_t* perm,
                     const uint8_t* bad, const double* mu, const DmmaParams& P, double* Y,
                     double* h, double* g, cudaStream_t s) {
    const uint64_t blocks = (n_pad * 32 + 255) / 256;
    pack_dmma_kernel<<<(unsigned)blocks, 256, 0, s>>>(X, n, n_pad, perm, bad, mu, P, Y, h, g);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

int launch_pack16(const float* Y32, const float* Yerr, uint64_t n, uint64_t n_pad,
                  const uint32_t* perm, const uint8_t* bad, const ScreenParams& P, void* Q,
                  void* Aug, float* beta, float* Xf, float* rad, cudaStream_t s) {
    if (n_pad % 32) return set_error(EJOIN_EINTERNAL, "pack16: rows not padded");
    const uint64_t blocks = (n_pad + 255) / 256;  // 8 warps x 32 rows per block
    if (P.fmt == Fmt::BF16)
        pack16_kernel<Fmt::BF16><<<(unsigned)blocks, 256, 0, s>>>(Y32, n, n_pad, perm, bad, Yerr,
                                                                  P, (uint16_t*)Q, (uint16_t*)Aug,
                                                                  beta, Xf, rad);
    else if (P.fmt == Fmt::FP16)
        pack16_kernel<Fmt::FP16><<<(unsigned)blocks, 256, 0, s>>>(Y32, n, n_pad, perm, bad, Yerr,
                                                                  P, (uint16_t*)Q, (uint16_t*)Aug,
                                                                  beta, Xf, rad);
    else
        return set_error(EJOIN_EINTERNAL, "pack16: bad format");
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

int launch_pack8(const float* Y32, const float* Yerr, uint64_t n, uint64_t n_pad,
                 const uint32_t* perm, const uint8_t* bad, const ScreenParams& P, uint8_t* Q,
                 void* Aug, float* beta, float* sig, float* Xf, float* rad, float* tsig,
                 uint16_t* Xh, float* radh, cudaStream_t s) {
    if (n_pad % 128) return set_error(EJOIN_EINTERNAL, "pack8: rows not padded");
    if (P.d > 32u * PACK8_MAXV) return set_error(EJOIN_EUNSUPPORTED, "FP8 screen supports d <= %d", 32 * PACK8_MAXV);
    pack8_kernel<<<(unsigned)((n_pad + 255) / 256), 256, 0, s>>>(Y32, n, n_pad, perm, bad, Yerr, P,
                                                                 Q, (uint16_t*)Aug, beta, sig, Xf, rad,
                                                                 Xh, radh);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    tile_min_sigma_kernel<<<(unsigned)(n_pad / 128), 128, 0, s>>>(sig, n_pad / 128, tsig);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

int launch_chunk_max(const float* beta, uint64_t n_pad, float* cmax, cudaStream_t s) {
    if (n_pad % 32) return set_error(EJOIN_EINTERNAL, "chunk max: rows not padded");
    if (n_pad == 0) return EJOIN_OK;
    chunk_max_kernel<<<(unsigned)((n_pad + 255) / 256), 256, 0, s>>>(beta, n_pad, cmax);
    EJ_CUDA(cudaGetLastError());
    note_launch();
    return EJOIN_OK;
}

}  // namespace ejoin
