// api.cu -- the C ABI of libejoin.so and the join driver.
//
// Re-designs the reference driver GPUJoinMainBruteForce (gpu_join.cu:210-322):
// the reference uploads the padded dataset, optionally converts it, computes
// chunked norms, launches one kernel chosen by searchMode, synchronises and
// copies one 64-bit counter back -- never zeroing the counter, never freeing
// device memory and exiting on an unknown mode.  Here the driver
//   1. places the points in device memory (host or device input),
//   2. runs the chosen exact pipeline:
//        FP64_DIRECT  exact FP64 tiles (the arbiter)
//        FP64_DMMA    FP64 Gram screen + band recheck
//        BF16/FP16    centre, scale, pack; tcgen05 Gram screen + band recheck
//      optionally behind the learned tile-pair pruning (k_learn.cu),
//   3. re-runs the screen with a larger band queue if it overflowed,
//   4. returns per-point counts and their total,
// with status codes instead of exits and all scratch freed on return.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <set>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "ejoin_internal.cuh"
#include "ejoin_testing.h"

namespace ejoin {

// ------------------------------------------------------------- errors --

static thread_local int t_status = 0;
static thread_local char t_msg[2048] = "";

int set_error(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_msg, sizeof t_msg, fmt, ap);
    va_end(ap);
    t_status = status;
    return status;
}

int cuda_error(cudaError_t e, const char* what, const char* file, int line) {
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? EJOIN_ENOMEM : EJOIN_ECUDA,
                     "%s failed (%s:%d): %s", what, file, line, cudaGetErrorString(e));
}

static thread_local uint64_t t_launches = 0;
void note_launch(uint64_t k) { t_launches += k; }
uint64_t launches_so_far() { return t_launches; }

void clear_error() {
    t_status = 0;
    t_msg[0] = 0;
}

// ------------------------------------------------------- scratch pool --

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pools[kMaxDevices] = {};
thread_local cudaMemPool_t t_pool = nullptr;
std::atomic<uint64_t> g_fail_at{0};
std::atomic<uint64_t> g_gram_timeout{0};

// The library's pool on device dev: device-local memory, freed blocks kept
// for the rest of a call (release threshold: unlimited; CallScope trims it).
int library_pool(int dev, cudaMemPool_t* out) {
    if (dev < 0 || dev >= kMaxDevices) return set_error(EJOIN_EINVAL, "device ordinal %d unsupported", dev);
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pools[dev]) {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        EJ_CUDA(cudaMemPoolCreate(&p, &props));
        uint64_t thr = UINT64_MAX;
        EJ_CUDA(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &thr));
        g_pools[dev] = p;
    }
    *out = g_pools[dev];
    return EJOIN_OK;
}
}  // namespace

cudaMemPool_t current_pool() { return t_pool; }

int CallScope::enter(int dev, cudaStream_t stream, bool keep_scratch) {
    EJ_TRY(library_pool(dev, &pool));
    prev = t_pool;
    t_pool = pool;
    s = stream;
    keep = keep_scratch;
    uint64_t zero = 0;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReservedMemHigh, &zero);
    return EJOIN_OK;
}

uint64_t CallScope::peak_reserved() const {
    uint64_t v = 0;
    if (pool) cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemHigh, &v);
    return v;
}

CallScope::~CallScope() {
    if (!pool) return;
    // every buffer of the call was freed on s (stream order) before this
    // runs; once s is idle the pool holds no live allocation of this call
    if (cudaStreamSynchronize(s) != cudaSuccess) cudaGetLastError();
    if (!keep) cudaMemPoolTrimTo(pool, 0);
    t_pool = prev;
}

void inject_alloc_failure(uint64_t k) { g_fail_at.store(k); }

bool alloc_should_fail() {
    uint64_t v = g_fail_at.load();
    while (v) {
        if (g_fail_at.compare_exchange_weak(v, v - 1)) return v == 1;
    }
    return false;
}

void inject_gram_timeout(uint64_t ns) { g_gram_timeout.store(ns); }
uint64_t take_gram_timeout() { return g_gram_timeout.exchange(0); }

// ------------------------------------------------------- host buffers --

namespace {
std::mutex g_host_mu;
std::set<void*> g_pinned;
}  // namespace

void* host_alloc(size_t bytes) {
    int count = 0;
    if (cudaGetDeviceCount(&count) == cudaSuccess && count > 0) {
        void* p = nullptr;
        if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) == cudaSuccess && p) {
            std::lock_guard<std::mutex> lk(g_host_mu);
            g_pinned.insert(p);
            return p;
        }
    }
    cudaGetLastError();
    return malloc(bytes);
}

void host_free(void* p) {
    if (!p) return;
    {
        std::lock_guard<std::mutex> lk(g_host_mu);
        auto it = g_pinned.find(p);
        if (it != g_pinned.end()) {
            g_pinned.erase(it);
            cudaFreeHost(p);
            return;
        }
    }
    free(p);
}

// ---------------------------------------------------------- threshold --

// Largest double T with sqrt(T) <= eps.  Correctly rounded sqrt is monotone,
// so sqrt(d2) <= eps (the reference predicate, kernel_join.cu:194) is
// exactly d2 <= T.  NaN eps -> NaN, eps < 0 -> -inf, +inf -> +inf.
double threshold(double eps) {
    if (isnan(eps)) return NAN;
    if (eps < 0.0) return -INFINITY;
    if (isinf(eps)) return INFINITY;
    double t = eps * eps;
    if (isinf(t)) t = 1.7976931348623157e308;
    while (t > 0.0 && sqrt(t) > eps) t = nextafter(t, 0.0);
    for (;;) {
        const double up = nextafter(t, INFINITY);
        if (isinf(up) || !(sqrt(up) <= eps)) break;
        t = up;
    }
    return t;
}

// Bounds of the oracle's rounding: d2 computed by the reference arithmetic
// satisfies |d2 - delta^2| <= c_o delta^2 + a_o for the exact squared
// distance delta^2 ((d+2) roundings of at most 2^-53 each, plus subnormal
// absolute error).  Pairs with delta^2 <= Tlo certainly satisfy d2 <= T;
// pairs with delta^2 > Thi certainly do not.
void oracle_band(double T, uint32_t d, double* Tlo, double* Thi) {
    const double co = (d + 4) * kU * 1.0001;
    const double ao = (d + 2) * 4.9406564584124654e-324 * 2.0;
    double lo = (T - ao) / (1.0 + co) * (1.0 - 4 * kU);
    double hi = (T + ao) / (1.0 - co) * (1.0 + 4 * kU);
    *Tlo = lo > 0.0 ? lo : 0.0;
    *Thi = hi;
}

// ------------------------------------------------------------- tracing --

// NVTX range over one phase of a join (prep, train, order, pack, gram,
// recheck), visible in Nsight Systems / Compute timelines; a no-op unless a
// tool is attached.  The phases' GPU times are also in ejoin_stats.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// ------------------------------------------------------------ devices --

struct DeviceScope {
    int prev = -1;
    int enter(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            cudaGetLastError();
            prev = -1;
        }
        EJ_CUDA(cudaSetDevice(dev));
        return EJOIN_OK;
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

static int check_device(int dev, int* sms) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        return set_error(EJOIN_ENODEV, "no CUDA device available (%s)",
                         e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
    }
    if (dev < 0 || dev >= count) return set_error(EJOIN_EINVAL, "device %d out of range (%d devices)", dev, count);
    cudaDeviceProp p;
    EJ_CUDA(cudaGetDeviceProperties(&p, dev));
    if (p.major != 10 || p.minor != 3)
        return set_error(EJOIN_ENODEV,
                         "device %d is sm_%d%d; libejoin.so is built for sm_103a (GB300) only", dev,
                         p.major, p.minor);
    *sms = p.multiProcessorCount;
    return EJOIN_OK;
}

static bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Compact n x d rows (row stride ld) into device memory.  With `defer`, dense
// rows in pinned host memory (64 MB or more) are not copied here: *defer
// describes them and the copy is left to the centring pass, which overlaps
// it with its own work (*deferred = true).
static int stage_points(const double* points, uint64_t n, uint32_t d, uint64_t ld, DBuf<double>& buf,
                        const double** Xout, cudaStream_t s, StageCopy* defer = nullptr,
                        bool* deferred = nullptr) {
    if (deferred) *deferred = false;
    const bool dev = is_device_ptr(points);
    if (dev && ld == d) {
        *Xout = points;
        return EJOIN_OK;
    }
    EJ_TRY(buf.alloc(n * d, s, "points"));
    if (defer && !dev && ld == d && n * d * sizeof(double) >= (64ull << 20)) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, points) == cudaSuccess && a.type == cudaMemoryTypeHost &&
            a.devicePointer) {
            *defer = StageCopy{points, (const double*)a.devicePointer};
            *deferred = true;
            *Xout = buf.p;
            return EJOIN_OK;
        }
        cudaGetLastError();
    }
    if (ld == d) {
        EJ_CUDA(cudaMemcpyAsync(buf.p, points, n * d * sizeof(double),
                                dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    } else {
        EJ_CUDA(cudaMemcpy2DAsync(buf.p, d * sizeof(double), points, ld * sizeof(double),
                                  d * sizeof(double), n,
                                  dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    }
    *Xout = buf.p;
    return EJOIN_OK;
}

// ---------------------------------------------------------- pipelines --

struct Join {
    cudaStream_t s;
    int sms;
    const double* X;  // n x d, device
    uint64_t n;
    uint32_t d;
    double eps;
    double T;
    ejoin_options opt;
    ejoin_stats* st;
    int32_t* counts;         // device, >= n_pad entries, packed-row order
    const uint32_t* perm;    // packed row -> original row (null = identity)
    const Emit* em = nullptr;  // neighbour-list emission (null: counts only)
    const StageCopy* stage = nullptr;  // X still to be copied (by the centring pass)
};

static uint64_t round_up(uint64_t v, uint64_t m) { return (v + m - 1) / m * m; }

static uint64_t band_budget(uint64_t want) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return want;
    }
    const uint64_t maxe = (uint64_t)(fr / 4) / sizeof(BandPair);
    return std::min(want, std::max<uint64_t>(maxe, 1u << 20));
}

// Runs `screen` (which fills counts and the band queue), re-running it with a
// larger queue on overflow, then `recheck` resolves the band exactly.  The
// queue holds `unit` BandPair-sized words per entry: pairs (unit 1) or band
// records (unit 2, with the pair count in DevStatus::band_pairs); capacities
// are in pairs.
template <typename Screen, typename Recheck>
static int screen_and_recheck(Join& J, uint64_t cap0, Screen&& screen, Recheck&& recheck,
                              uint64_t n_pad, EventTimer& tg, EventTimer& tr, uint32_t unit = 1) {
    DBuf<BandPair> band;
    DBuf<DevStatus> dst;
    EJ_TRY(dst.alloc(1, J.s, "status"));
    uint64_t cap = band_budget(J.opt.band_capacity ? J.opt.band_capacity : cap0);
    for (int attempt = 0;; ++attempt) {
        EJ_TRY(band.alloc(cap, J.s, "band queue"));
        EJ_TRY(dst.zero(J.s));
        if (const uint64_t ns = unit == 2 ? take_gram_timeout() : 0) {
            // test hook: short deadline, producer withholds its first stage
            const uint32_t one = 1;
            EJ_CUDA(cudaMemcpyAsync(&dst.p->wait_ns, &ns, sizeof ns, cudaMemcpyHostToDevice, J.s));
            EJ_CUDA(cudaMemcpyAsync(&dst.p->withhold, &one, sizeof one, cudaMemcpyHostToDevice, J.s));
            EJ_CUDA(cudaStreamSynchronize(J.s));
        }
        EJ_CUDA(cudaMemsetAsync(J.counts, 0, n_pad * sizeof(int32_t), J.s));
        tg.start(J.s);
        {
            NvtxRange nr("ejoin:gram");
            EJ_TRY(screen(band.p, cap / unit, dst.p));
        }
        tg.stop(J.s);
        DevStatus h;
        EJ_CUDA(cudaMemcpyAsync(&h, dst.p, sizeof h, cudaMemcpyDeviceToHost, J.s));
        EJ_CUDA(cudaStreamSynchronize(J.s));
        if (h.timeout)
            return set_error(EJOIN_ETIMEOUT, "Gram kernel: a bounded device wait expired (site %u)", h.where);
        if (h.band_count <= cap / unit) {
            const uint64_t pairs = unit == 1 ? h.band_count : h.band_pairs;
            tr.start(J.s);
            {
                NvtxRange nr("ejoin:recheck");
                EJ_TRY(recheck(band.p, h.band_count, pairs, dst.p));
            }
            tr.stop(J.s);
            EJ_CUDA(cudaMemcpyAsync(&h, dst.p, sizeof h, cudaMemcpyDeviceToHost, J.s));
            EJ_CUDA(cudaStreamSynchronize(J.s));
            J.st->band_pairs = pairs;
            J.st->band_hits = h.band_hits;
            J.st->reserved[0] = (double)h.exact_rechecks;
            J.st->reserved[3] = unit == 2 ? (double)h.band_records : 0.0;
            J.st->ms_gram = tg.ms();
            J.st->ms_recheck = tr.ms();
            return EJOIN_OK;
        }
        J.st->band_overflows++;
        const uint64_t want = (h.band_count + h.band_count / 16 + 1024) * unit;
        const uint64_t got = band_budget(want);
        if (got < want || attempt >= 3)
            return set_error(EJOIN_ENOMEM, "band queue needs %llu entries; device memory allows %llu",
                             (unsigned long long)want, (unsigned long long)got);
        cap = want;
    }
}

static int run_direct(Join& J) {
    EventTimer t;
    EJ_CUDA(cudaMemsetAsync(J.counts, 0, J.n * sizeof(int32_t), J.s));
    t.start(J.s);
    EJ_TRY(launch_direct_selfjoin(J.X, J.n, J.d, J.T, J.counts, J.em, J.s));
    t.stop(J.s);
    J.st->ms_gram = t.ms();
    const double pairs = (double)J.n * (double)(J.n + 1) / 2.0;
    J.st->gram_flops = 3.0 * J.d * pairs;
    J.st->precision = EJOIN_FP64_DIRECT;
    return EJOIN_OK;
}

static int run_dmma(Join& J) {
    // pair emission runs on the exact arbiter (the DMMA epilogue only counts)
    if (J.em) return run_direct(J);
    EventTimer tp, tg, tr;
    tp.start(J.s);
    DBuf<uint8_t> bad;
    DBuf<double> mu;
    EJ_TRY(bad.alloc(J.n, J.s, "row flags"));
    EJ_TRY(mu.alloc(J.d, J.s, "mean"));
    CenterStats cs;
    EJ_TRY(launch_center_stats(J.X, J.n, J.d, bad.p, mu.p, nullptr, nullptr, &cs, J.s));
    DmmaParams P;
    P.d = J.d;
    P.dp = (uint32_t)round_up(J.d, 32);
    oracle_band(J.T, J.d, &P.Tlo, &P.Thi);
    P.sTlo = sqrt(P.Tlo) * (1 - 4 * kU);
    P.sThi = sqrt(P.Thi) * (1 + 4 * kU);
    P.crel = 2.0 * (P.dp + 8) * kU;
    const uint64_t n_pad = round_up(J.n, 64);
    DBuf<double> Y, h, g;
    EJ_TRY(Y.alloc(n_pad * P.dp, J.s, "centred FP64 rows"));
    EJ_TRY(h.alloc(n_pad, J.s, "in thresholds"));
    EJ_TRY(g.alloc(n_pad, J.s, "out thresholds"));
    EJ_TRY(launch_pack_dmma(J.X, J.n, n_pad, J.perm, bad.p, mu.p, P, Y.p, h.p, g.p, J.s));
    tp.stop(J.s);
    J.st->ms_prep = tp.ms();
    const uint64_t nT = n_pad / 64;
    J.st->tile_pairs_total = nT * (nT + 1) / 2;
    J.st->tile_pairs_run = J.st->tile_pairs_total;
    J.st->gram_flops = 2.0 * P.dp * 64.0 * 64.0 * (double)J.st->tile_pairs_run;
    J.st->precision = EJOIN_FP64_DMMA;
    auto screen = [&](BandPair* band, uint64_t cap, DevStatus* st) {
        return launch_dmma_join(Y.p, n_pad, P.dp, h.p, g.p, J.counts, band, cap, st, J.s);
    };
    auto recheck = [&](const BandPair* band, uint64_t nb, uint64_t, DevStatus* st) {
        return launch_band_recheck(J.X, J.n, J.d, J.perm, J.T, band, nb, J.counts, st, J.s);
    };
    return screen_and_recheck(J, std::max<uint64_t>(1u << 20, J.n), screen, recheck, n_pad, tg, tr);
}

// Learned ordering: projection P (given or trained on the GPU), its certified
// spectral-norm bound sigma, the permutation into projected order and the
// boxes of the 128-row tiles.  A tile pair is skipped when the squared gap of
// its boxes exceeds sigma^2 * T_hi: then every pair in it has
// delta^2 >= gap^2 / sigma^2 > T_hi, i.e. d2 > T.
struct Learned {
    DBuf<uint32_t> perm;
    LearnedBoxes boxes;
    float thr = 0.0f;
    uint32_t k = 0;
};

static int prepare_learned(Join& J, const float* Y32, const float* Yerr, const uint8_t* bad,
                           uint64_t n_pad, Learned& L, TrainResult* trained = nullptr,
                           double ms_trained = 0.0) {
    const uint32_t k = J.opt.proj_k;
    if (k == 0 || k > 16) return set_error(EJOIN_EINVAL, "proj_k must be in 0..16 (got %u)", k);
    EventTimer tt, to;
    std::vector<float> P;
    double sigma = 0.0;
    tt.start(J.s);
    if (J.opt.projection) {
        P.assign(J.opt.projection, J.opt.projection + (size_t)k * J.d);
        EJ_TRY(cert_spectral_norm(P.data(), k, J.d, &sigma));
    } else if (trained) {
        // trained already, overlapping the centring pass (run_screen16)
        P.swap(trained->P);
        sigma = trained->sigma_cert;
    } else {
        TrainResult tr;
        EJ_TRY(train_projection_dev(Y32, bad, training_rows(J.n), J.d, J.eps, k, J.opt.train_pairs,
                                    J.opt.train_steps, J.opt.seed, J.opt.order == EJOIN_ORDER_LEAD,
                                    J.s, tr));
        P.swap(tr.P);
        sigma = tr.sigma_cert;
    }
    tt.stop(J.s);
    to.start(J.s);
    DBuf<float> Pd;
    EJ_TRY(Pd.alloc(P.size(), J.s, "projection"));
    EJ_CUDA(cudaMemcpyAsync(Pd.p, P.data(), P.size() * sizeof(float), cudaMemcpyHostToDevice, J.s));
    // pmax >= max_a |P_a| (products of FP32 values are exact in FP64; the
    // relative margin covers the summation and square-root roundings)
    double pm = 0.0;
    for (uint32_t a = 0; a < k; ++a) {
        double s2 = 0.0;
        for (uint32_t c = 0; c < J.d; ++c) s2 += (double)P[(size_t)a * J.d + c] * P[(size_t)a * J.d + c];
        pm = std::max(pm, sqrt(s2) * (1.0 + (J.d + 4) * kU));
    }
    float pmax = (float)pm;
    if ((double)pmax < pm) pmax = nextafterf(pmax, INFINITY);
    if (!std::isfinite(pmax)) return set_error(EJOIN_EINVAL, "projection has non-finite entries");
    EJ_TRY(learned_order(Y32, Yerr, bad, J.n, n_pad, J.d, Pd.p, k, pmax,
                         J.opt.order == EJOIN_ORDER_LEAD, L.perm, &L.boxes, J.s));
    to.stop(J.s);
    double Tlo, Thi;
    oracle_band(J.T, J.d, &Tlo, &Thi);
    // FP32 threshold rounded up: the box-gap test then never prunes a pair
    // that the exact bound would keep
    const double thr = Thi * sigma * sigma * (1.0 + 32 * kU);
    float tf = (float)thr;
    if ((double)tf < thr) tf = nextafterf(tf, INFINITY);
    L.thr = tf;
    L.k = k;
    J.perm = L.perm.p;
    J.st->sigma_cert = sigma;
    J.st->ms_train = trained ? ms_trained : tt.ms();
    J.st->ms_order = to.ms();
    return EJOIN_OK;
}

// Global power-of-two scale of the centred data for the 16-bit operands.
static double screen_scale(Fmt f, double maxabs, uint32_t d) {
    // BF16 / FP8: max |z| <= 1 (FP8 rows get their own scale on top);
    // FP16: max |z|^2 <= 2^12 so that norms and margins stay in range
    if (!(maxabs > 0.0) || !isfinite(maxabs)) return 1.0;
    double target = (f == Fmt::FP16) ? 64.0 / sqrt((double)d) : 1.0;
    int e = (int)floor(log2(target / maxabs));
    e = std::max(-1000, std::min(1000, e));
    return ldexp(1.0, e);
}

// Parameters of the 16-bit / FP8 screen for data with max |centred coord|
// maxabs (see pack16_kernel / pack8_kernel for the bounds they feed).
static ScreenParams screen_params(Fmt fmt, bool split, uint32_t d, double maxabs, double T,
                                  double acc_bound_scale, double* kprod_out) {
    ScreenParams P;
    const bool fp8 = (fmt == Fmt::E4M3);
    P.fmt = fmt;
    P.split = split ? 1 : 0;
    P.d = d;
    P.dp = (uint32_t)round_up(d, fp8 ? 128 : 64);
    P.width = P.dp * (split ? 2 : 1);
    P.scale = screen_scale(fmt, maxabs, d);
    double Tlo, Thi;
    oracle_band(T, d, &Tlo, &Thi);
    const double s2 = P.scale * P.scale;
    // Every finite pair has s_q = |q_i - q_j|^2 <= 4 max|q|^2 (<= 2^14 for FP16
    // by the choice of scale, <= 4d for BF16 / FP8): capping T far above that
    // keeps both tests exact while bounding the margins in the operand range.
    const double cap_t = (fmt == Fmt::FP16) ? 32768.0 : 1.152921504606846976e18;
    P.Tlo = std::min(Tlo * s2, cap_t);
    P.Thi = std::min(Thi * s2, cap_t);
    P.sTlo = sqrt(P.Tlo) * (1 - 4 * kU);
    P.sThi = sqrt(P.Thi) * (1 + 4 * kU);
    const double kprod = (split ? 3.0 : 1.0) * P.dp + 16.0;  // + the aug K = 16 step
    // Accumulation bound.  Model of one tcgen05.mma of K_t products (K_t = 16
    // for the 16-bit kinds, 32 for E4M3) into an FP32 accumulator:
    //   S_t = S_{t-1} + sum_t p + e_t,  |e_t| <= K_t 2^-22 (|S_{t-1}| + sum_t |p|),
    // twice the error of K_t truncating FP32 additions, each charged with the
    // magnitude of all that was accumulated up to the end of the instruction;
    // 16 2^-22 of the total magnitude more covers the final value.  MMAs into
    // one accumulator act in issue order (D = A B + D), and the issuer
    // (k_umma.cu) orders them by magnitude: with the split, the hi*lo and
    // lo*hi products of the first K-slab (128 products, everything so far
    // <= L_ij = sum |hi_i lo_j| + |lo_i hi_j|), then every other data product
    // (<= L_ij + H_ij <= a_i a_j, a = |(|hi| + |lo|)|), then the aug step
    // (<= a_i a_j + |alpha_i| + |alpha_j|).  So
    //   |err| <= 2^-22 [128 L_ij + c_h a_i a_j + 32 (|alpha_i| + |alpha_j|)],
    //   c_h = 64 + 192 (slabs - 1) + 16 + 16 with the split, dp + 16 + 16 without,
    // and a_i a_j <= (a_i^2 + a_j^2) / 2, L_ij <= a_i l_j + l_i a_j
    // <= 2^-9 (a_i^2 + a_j^2) / 2 + 2^9 (l_i^2 + l_j^2) / 2 split it into the
    // per-row terms of acc_margin2.  (Charging every product with the total
    // instead gives the coarser (kprod + 16) 2^-22 (a_i a_j + |alpha_i| +
    // |alpha_j|), which this bound never exceeds.)
    const double scale_opt = acc_bound_scale > 0 ? acc_bound_scale : 1.0;
    const double slabs = P.dp / 64.0;
    const double c_h = split ? 96.0 + 192.0 * (slabs - 1.0) : P.dp + 32.0;
    P.cacc_a = scale_opt * c_h * ldexp(1.0, -22);
    P.cacc_l = split ? scale_opt * 128.0 * ldexp(1.0, -22) : 0.0;
    P.cacc_al = scale_opt * 32.0 * ldexp(1.0, -22);
    P.absacc = (kprod + 16.0) * ldexp(1.0, -125);
    P.inv_in_pos = nextafter(1.0 / (2.0 * (1.0 - P.cacc_al)), INFINITY);
    P.inv_in_neg = nextafter(1.0 / (2.0 * (1.0 + P.cacc_al)), 0.0);
    P.flush_err = nextafter(ldexp(1.0, -126) * sqrt((double)d), INFINITY);
    P.clamp_lo = (fmt == Fmt::FP16) ? -16384.0 : -kTwo100;
    *kprod_out = kprod;
    return P;
}

// One packed operand side: operands, aug rows, margins, FP32 coordinates.
struct PackedSide {
    uint64_t n_pad = 0;
    DBuf<uint16_t> Q, Aug;
    DBuf<uint8_t> Q8;
    DBuf<float> beta, cmax, Xf, rad, sig, tsig, radh;
    DBuf<uint16_t> Xh;  // FP16 copy of Xf (FP8 screen, rows longer than 64)
    const void* operands(const ScreenParams& P) const {
        return P.fmt == Fmt::E4M3 ? (const void*)Q8.p : (const void*)Q.p;
    }
};

static int pack_side(const float* Y32, const float* Yerr, const uint8_t* bad, uint64_t n,
                     uint64_t n_pad, const uint32_t* perm, const ScreenParams& P, PackedSide& S,
                     cudaStream_t s) {
    const bool fp8 = P.fmt == Fmt::E4M3;
    S.n_pad = n_pad;
    if (fp8) EJ_TRY(S.Q8.alloc(n_pad * P.width, s, "packed FP8 operands"));
    else EJ_TRY(S.Q.alloc(n_pad * P.width, s, "packed operands"));
    EJ_TRY(S.Aug.alloc(n_pad * 32, s, "aug operands"));
    EJ_TRY(S.beta.alloc(n_pad, s, "out margins"));
    EJ_TRY(S.cmax.alloc(n_pad / 32, s, "chunk margins"));
    EJ_TRY(S.Xf.alloc(n_pad * P.d, s, "FP32 coordinates"));
    EJ_TRY(S.rad.alloc(n_pad, s, "FP32 radii"));
    if (fp8) {
        EJ_TRY(S.sig.alloc(n_pad, s, "row scales"));
        EJ_TRY(S.tsig.alloc(n_pad / 128, s, "tile scales"));
        // the wide E4M3 band is first rechecked on FP16 copies (half the
        // bytes of the FP32 rows); the warp recheck kernel (d > 64) uses them
        if (P.d > 64) {
            EJ_TRY(S.Xh.alloc(n_pad * P.d, s, "FP16 coordinates"));
            EJ_TRY(S.radh.alloc(n_pad, s, "FP16 radii"));
        }
        EJ_TRY(launch_pack8(Y32, Yerr, n, n_pad, perm, bad, P, S.Q8.p, S.Aug.p, S.beta.p, S.sig.p,
                            S.Xf.p, S.rad.p, S.tsig.p, S.Xh.p, S.radh.p, s));
    } else {
        EJ_TRY(launch_pack16(Y32, Yerr, n, n_pad, perm, bad, P, S.Q.p, S.Aug.p, S.beta.p, S.Xf.p,
                             S.rad.p, s));
    }
    return launch_chunk_max(S.beta.p, n_pad, S.cmax.p, s);
}

// L owns the permutation that J.perm points to; it must outlive the final
// scatter of the counts, so the caller keeps it.
static int run_screen16(Join& J, Fmt fmt, bool split, Learned& L) {
    EventTimer tp, tg, tr;
    tp.start(J.s);
    DBuf<uint8_t> bad;
    DBuf<double> mu;
    EJ_TRY(bad.alloc(J.n, J.s, "row flags"));
    EJ_TRY(mu.alloc(J.d, J.s, "mean"));
    DBuf<float> Y32, Yerr;
    EJ_TRY(Y32.alloc(J.n * J.d, J.s, "FP32 centred points"));
    EJ_TRY(Yerr.alloc(J.n, J.s, "centring error bounds"));
    CenterStats cs;
    // Projection training samples the first training_rows(n) rows; it starts
    // on a stream of its own as soon as those rows are centred, so with a
    // staged (pinned host) input it runs while the rest is still copied.
    const bool train = J.opt.proj_k && L.k == 0 && !J.opt.projection;
    TrainResult trained;
    bool have_trained = false;
    double ms_train = 0.0;
    const uint64_t nt = training_rows(J.n);
    // end of the centring pass on J.s (recorded when the hook starts: every
    // centring launch is enqueued by then), so that ms_prep leaves the
    // overlapped training out
    EventTimer tc;
    bool centred_marked = false;
    PrefixHook hook = [&](cudaEvent_t ready) -> int {
        if (J.opt.proj_k == 0 || J.opt.proj_k > 16)
            return set_error(EJOIN_EINVAL, "proj_k must be in 0..16 (got %u)", J.opt.proj_k);
        tc.stop(J.s);
        centred_marked = true;
        cudaStream_t ts = nullptr;
        EJ_CUDA(cudaStreamCreateWithFlags(&ts, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
        } guard{ts};
        EJ_CUDA(cudaStreamWaitEvent(ts, ready, 0));
        NvtxRange nr("ejoin:train");
        EventTimer tt;
        tt.start(ts);
        EJ_TRY(train_projection_dev(Y32.p, bad.p, nt, J.d, J.eps, J.opt.proj_k, J.opt.train_pairs,
                                    J.opt.train_steps, J.opt.seed, J.opt.order == EJOIN_ORDER_LEAD,
                                    ts, trained));
        tt.stop(ts);
        ms_train = tt.ms();
        have_trained = true;
        return EJOIN_OK;
    };
    {
        NvtxRange nr("ejoin:prep");
        EJ_TRY(launch_center_stats(J.X, J.n, J.d, bad.p, mu.p, Y32.p, Yerr.p, &cs, J.s, false,
                                   J.stage, nt, train && J.n >= 2 ? &hook : nullptr));
    }
    J.stage = nullptr;
    tp.stop(J.s);
    double ms_center = tp.ms();
    if (centred_marked) {
        float v = 0.f;
        cudaEventElapsedTime(&v, tp.a, tc.b);
        ms_center = v;
    }
    // The FP32 copies need the centred coordinates well inside the FP32 range:
    // squared norms of up to 2^27 coordinates must not overflow, and the
    // absolute error terms (2^-126 per flushed coordinate, underflow of FP32
    // norms) must stay negligible.  Other data takes the (equally exact) FP64
    // DMMA screen.
    const double maxabs = cs.maxy;
    const bool fp32_ok = !cs.range && (maxabs == 0.0 ? !cs.flushed
                                                     : (maxabs >= 0x1p-50 && maxabs <= 0x1p50));
    if (!fp32_ok) return run_dmma(J);
    // rows padded to whole 128 x 256 blocks of the Gram kernel
    const uint64_t n_pad = round_up(J.n, 256);
    // a second pass of the same join (pair emission) reuses the ordering
    if (J.opt.proj_k && L.k == 0) {
        NvtxRange nr("ejoin:order");
        EJ_TRY(prepare_learned(J, Y32.p, Yerr.p, bad.p, n_pad, L, have_trained ? &trained : nullptr,
                               ms_train));
    }
    tp.start(J.s);
    const bool fp8 = (fmt == Fmt::E4M3);
    double kprod = 0;
    const ScreenParams P = screen_params(fmt, split, J.d, maxabs, J.T, J.opt.acc_bound_scale, &kprod);
    PackedSide side;
    {
        NvtxRange nr("ejoin:pack");
        EJ_TRY(pack_side(Y32.p, Yerr.p, bad.p, J.n, n_pad, J.perm, P, side, J.s));
    }
    tp.stop(J.s);
    J.st->ms_prep = ms_center + tp.ms();
    const uint64_t nT = n_pad / 128;
    DBuf<uint2> work;
    uint64_t nwork = 0;
    EventTimer tw;
    tw.start(J.s);
    uint64_t ntiles = 0;
    const uint64_t nTa = (J.n + 127) / 128;
    EJ_TRY(build_worklist(nT, nTa, L.k ? &L.boxes : nullptr, L.thr, work, &nwork, &ntiles, J.s));
    tw.stop(J.s);
    J.st->ms_order += tw.ms();
    J.st->tile_pairs_total = nTa * (nTa + 1) / 2;
    J.st->tile_pairs_run = ntiles;
    J.st->reserved[1] = (double)nwork;
    J.st->gram_flops = 2.0 * kprod * 128.0 * 256.0 * (double)nwork;
    J.st->precision = fp8 ? EJOIN_FP8_E4M3
                          : (fmt == Fmt::FP16 ? EJOIN_FP16 : (split ? EJOIN_BF16_SPLIT : EJOIN_BF16));
    const void* Qp = side.operands(P);
    auto screen = [&](BandPair* band, uint64_t cap, DevStatus* st) {
        const GramSide gs{Qp, side.Aug.p, n_pad};
        return launch_gram16(gs, gs, P, work.p, nwork, side.cmax.p, side.beta.p, side.tsig.p,
                             side.sig.p, false,
                             J.counts, reinterpret_cast<BandRec*>(band), cap, st, J.em, J.sms,
                             J.s);
    };
    Recheck32 R;
    R.Xf = R.Xfb = side.Xf.p;
    R.rad = R.radb = side.rad.p;
    R.Xh = R.Xhb = side.Xh.p;
    R.radh = R.radhb = side.radh.p;
    R.Xb = J.X;
    R.nb = J.n;
    R.permb = J.perm;
    R.sTlo = P.sTlo;
    R.sThi = P.sThi;
    R.c32 = (J.d + 8) * ldexp(1.0, -24) * 1.01;
    R.abs32 = (J.d + 8) * ldexp(1.0, -148);
    finish_recheck32(R);
    // band records -> pairs, then the FP32 pre-check / exact FP64 recheck
    auto recheck = [&](const BandPair* band, uint64_t nrec, uint64_t npairs, DevStatus* st) {
        if (npairs == 0) return EJOIN_OK;
        DBuf<BandPair> pairs;
        EJ_TRY(pairs.alloc(npairs, J.s, "band pairs"));
        EJ_TRY(launch_band_expand(reinterpret_cast<const BandRec*>(band), nrec, pairs.p, npairs,
                                  J.s));
        return launch_band_recheck2(J.X, J.n, J.d, J.perm, J.T, R, pairs.p, npairs, J.counts, st,
                                    J.em, J.s);
    };
    // First queue: sized from a systematic sample of the blocks (every
    // stride-th, about 8,192 of them, stride 64 to 256; counting records
    // only) when the list could produce more records than the minimum queue;
    // an overflow re-runs the whole screen with the exact size.  (A block
    // produces at most 128 rows x 8 chunks = 1024 records.)
    uint64_t cap_rec = 1u << 22;
    if (!J.opt.band_capacity && nwork * 1024 > cap_rec) {
        EventTimer te;
        te.start(J.s);
        DBuf<uint2> sw;
        DBuf<DevStatus> est;
        uint64_t ns = 0;
        const uint64_t stride = std::min<uint64_t>(256, std::max<uint64_t>(64, nwork / 8192));
        EJ_TRY(sample_worklist(work.p, nwork, stride, sw, &ns, J.s));
        EJ_TRY(est.alloc(1, J.s, "band estimate"));
        EJ_TRY(est.zero(J.s));
        const GramSide gs{Qp, side.Aug.p, n_pad};
        EJ_TRY(launch_gram16(gs, gs, P, sw.p, ns, side.cmax.p, side.beta.p, side.tsig.p,
                             side.sig.p, false, J.counts, nullptr, 0, est.p, nullptr, J.sms, J.s));
        DevStatus h;
        EJ_CUDA(cudaMemcpyAsync(&h, est.p, sizeof h, cudaMemcpyDeviceToHost, J.s));
        EJ_CUDA(cudaStreamSynchronize(J.s));
        te.stop(J.s);
        J.st->ms_order += te.ms();
        if (h.timeout)
            return set_error(EJOIN_ETIMEOUT, "Gram kernel: a bounded device wait expired (site %u)", h.where);
        const double scaled = (double)h.band_records * (double)nwork / (double)std::max<uint64_t>(ns, 1);
        cap_rec = std::max<uint64_t>(cap_rec, (uint64_t)(1.3 * scaled) + (1u << 20));
    }
    return screen_and_recheck(J, 2 * cap_rec, screen, recheck, n_pad, tg, tr, 2);
}

// AUTO (measured on GB300 over the benchmark shapes): FP16's 11-bit
// significand keeps the band narrow at a third of the split's MMA work for
// d <= 128; beyond that the FP32 accumulation term (proportional to K)
// dominates the bound and BF16 (wider range, no scaling limits) is as fast.
static int resolve_precision(int p, uint32_t d) {
    if (p == EJOIN_AUTO) return d <= 128 ? EJOIN_FP16 : EJOIN_BF16;
    return p;
}

// Neighbour-list request of self_join_impl: offsets [n + 1] and neighbors
// [capacity] (host or device; neighbors may be null: offsets only).  status
// becomes EJOIN_ENOMEM when capacity is below the total (lists not written).
struct ListsReq {
    uint64_t* offsets;
    uint32_t* neighbors;
    uint64_t capacity;
    int status = EJOIN_OK;
};

static int self_join_impl(const double* points, uint64_t n, uint32_t d, double eps,
                          const ejoin_options* opt_in, int32_t* counts_out, uint64_t* total_out,
                          ejoin_stats* stats_out, ListsReq* lists = nullptr) {
    ejoin_options opt;
    ejoin_default_options(&opt);
    if (opt_in) {
        if (opt_in->struct_size != sizeof(ejoin_options))
            return set_error(EJOIN_EINVAL, "ejoin_options.struct_size mismatch (%u != %zu)",
                             opt_in->struct_size, sizeof(ejoin_options));
        opt = *opt_in;
    }
    if (d == 0) return set_error(EJOIN_EINVAL, "dimension must be >= 1");
    if (n && !points) return set_error(EJOIN_EINVAL, "points is NULL");
    if (n > 0x7fffff00ull) return set_error(EJOIN_EUNSUPPORTED, "n = %llu exceeds 2^31 - 256", (unsigned long long)n);
    const uint64_t ld = opt.ld ? opt.ld : d;
    if (ld < d) return set_error(EJOIN_EINVAL, "row stride %llu < d %u", (unsigned long long)ld, d);
    if (opt.precision < EJOIN_FP64_DIRECT || opt.precision > EJOIN_AUTO)
        return set_error(EJOIN_EINVAL, "unknown precision mode %d", opt.precision);
    if (opt.acc_bound_scale < 1.0)
        return set_error(EJOIN_EINVAL, "acc_bound_scale must be >= 1 (got %g)", opt.acc_bound_scale);
    ejoin_stats stats;
    memset(&stats, 0, sizeof stats);
    stats.n = n;
    stats.d = d;
    DeviceScope ds;
    int sms = 0;
    EJ_TRY(check_device(opt.device, &sms));
    EJ_TRY(ds.enter(opt.device));
    cudaStream_t s = opt.stream ? (cudaStream_t)opt.stream : cudaStreamPerThread;
    CallScope scope;  // before every device buffer of the call
    EJ_TRY(scope.enter(opt.device, s, (opt.flags & EJOIN_FLAG_KEEP_SCRATCH) != 0));
    const bool out_dev = is_device_ptr(counts_out);
    const double T = threshold(eps);
    const uint64_t launches0 = launches_so_far();
    EventTimer tt;
    tt.start(s);

    Join J;
    J.s = s;
    J.sms = sms;
    J.n = n;
    J.d = d;
    J.eps = eps;
    J.T = T;
    J.opt = opt;
    J.st = &stats;
    J.perm = nullptr;
    DBuf<double> xbuf;
    DBuf<int32_t> cbuf;
    Learned learned;  // owns J.perm when the learned ordering is used
    const uint64_t n_pad = round_up(std::max<uint64_t>(n, 1), 256);  // padded rows of every screen
    EJ_TRY(cbuf.alloc(n_pad, s, "counts"));
    EJ_TRY(cbuf.zero(s));
    J.counts = cbuf.p;
    int prec = resolve_precision(opt.precision, d);
    stats.precision = prec;
    const bool run = n > 0 && !isnan(T) && T >= 0.0;
    auto run_once = [&]() -> int {
        switch (prec) {
            case EJOIN_FP64_DIRECT: return run_direct(J);
            case EJOIN_FP64_DMMA: return run_dmma(J);
            case EJOIN_FP16: return run_screen16(J, Fmt::FP16, false, learned);
            case EJOIN_BF16: return run_screen16(J, Fmt::BF16, false, learned);
            case EJOIN_BF16_SPLIT: return run_screen16(J, Fmt::BF16, true, learned);
            case EJOIN_FP8_E4M3: return run_screen16(J, Fmt::E4M3, false, learned);
            default: return set_error(EJOIN_EINVAL, "unknown precision %d", prec);
        }
    };
    StageCopy sc{};
    if (run) {
        if (isinf(T)) prec = EJOIN_FP64_DIRECT;  // every non-NaN pair counts: arbiter only
        // the 16-bit screens start with the centring pass, which takes over
        // the host-to-device copy of pinned input
        const bool screen16 = prec == EJOIN_FP16 || prec == EJOIN_BF16 ||
                              prec == EJOIN_BF16_SPLIT || prec == EJOIN_FP8_E4M3;
        bool deferred = false;
        EJ_TRY(stage_points(points, n, d, ld, xbuf, &J.X, s, screen16 ? &sc : nullptr, &deferred));
        J.stage = deferred ? &sc : nullptr;
        const int rc = run_once();
        if (J.stage) {
            // not taken over (an early failure): no pass may read X after this
            J.stage = nullptr;
            EJ_TRY(rc == EJOIN_OK ? set_error(EJOIN_EINTERNAL, "points were never staged") : rc);
        }
        EJ_TRY(rc);
    }
    DBuf<unsigned long long> tot;
    EJ_TRY(tot.alloc(1, s, "total"));
    EJ_TRY(tot.zero(s));
    EJ_TRY(sum_counts(J.counts, n, tot.p, s));
    if (counts_out && n) {
        if (J.perm) {
            if (out_dev) {
                EJ_TRY(scatter_counts(J.counts, J.perm, n, counts_out, s));
            } else {
                DBuf<int32_t> tmp;
                EJ_TRY(tmp.alloc(n, s, "scattered counts"));
                EJ_TRY(scatter_counts(J.counts, J.perm, n, tmp.p, s));
                EJ_CUDA(cudaMemcpyAsync(counts_out, tmp.p, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
                EJ_CUDA(cudaStreamSynchronize(s));
            }
        } else {
            EJ_CUDA(cudaMemcpyAsync(counts_out, J.counts, n * sizeof(int32_t),
                                    out_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
        }
    }
    unsigned long long total = 0;
    EJ_CUDA(cudaMemcpyAsync(&total, tot.p, sizeof total, cudaMemcpyDeviceToHost, s));
    if (lists) {
        // offsets from the counts (input order); the lists from a second pass
        // of the same join that emits its pairs (capacities: at most one
        // record or pair per counted pair)
        EJ_CUDA(cudaStreamSynchronize(s));
        DBuf<int32_t> corig;
        const int32_t* cin = J.counts;
        if (J.perm && n) {
            EJ_TRY(corig.alloc(n, s, "counts in input order"));
            EJ_TRY(scatter_counts(J.counts, J.perm, n, corig.p, s));
            cin = corig.p;
        }
        DBuf<unsigned long long> off;
        EJ_TRY(off.alloc(n + 1, s, "list offsets"));
        EJ_TRY(csr_offsets(cin, n, total, off.p, s));
        const bool off_dev = is_device_ptr(lists->offsets);
        EJ_CUDA(cudaMemcpyAsync(lists->offsets, off.p, (n + 1) * sizeof(uint64_t),
                                off_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
        if (lists->neighbors && lists->capacity < total) {
            lists->status = EJOIN_ENOMEM;
            set_error(EJOIN_ENOMEM, "neighbour buffer holds %llu of %llu entries",
                      (unsigned long long)lists->capacity, (unsigned long long)total);
        } else if (lists->neighbors && total > 0) {
            DBuf<BandRec> inq;
            DBuf<BandPair> pq;
            DBuf<unsigned long long> cnt;
            EJ_TRY(inq.alloc(total, s, "emitted records"));
            EJ_TRY(pq.alloc(total, s, "emitted pairs"));
            EJ_TRY(cnt.alloc(2, s, "emission counters"));
            EJ_TRY(cnt.zero(s));
            Emit em{inq.p, total, pq.p, total, cnt.p};
            J.em = &em;
            EJ_CUDA(cudaMemsetAsync(J.counts, 0, n_pad * sizeof(int32_t), s));
            EJ_TRY(run_once());
            J.em = nullptr;
            unsigned long long hc[2];
            EJ_CUDA(cudaMemcpyAsync(hc, cnt.p, sizeof hc, cudaMemcpyDeviceToHost, s));
            EJ_CUDA(cudaStreamSynchronize(s));
            if (hc[0] > total || hc[1] > total)
                return set_error(EJOIN_EINTERNAL, "neighbour lists: emission overflow");
            const bool nb_dev = is_device_ptr(lists->neighbors);
            DBuf<uint32_t> nbuf;
            uint32_t* nb = lists->neighbors;
            if (!nb_dev) {
                EJ_TRY(nbuf.alloc(total, s, "neighbour lists"));
                nb = nbuf.p;
            }
            EJ_TRY(csr_fill(off.p, n, total, inq.p, hc[0], pq.p, hc[1], J.perm, nb, s));
            if (!nb_dev)
                EJ_CUDA(cudaMemcpyAsync(lists->neighbors, nb, total * sizeof(uint32_t),
                                        cudaMemcpyDeviceToHost, s));
        }
        EJ_CUDA(cudaStreamSynchronize(s));
    }
    tt.stop(s);
    EJ_CUDA(cudaStreamSynchronize(s));
    stats.ms_total = tt.ms();
    stats.kernel_launches = launches_so_far() - launches0;
    stats.reserved[2] = (double)scope.peak_reserved();
    const double computed = (double)n * (double)n;
    stats.band_fraction = computed > 0 ? (double)stats.band_pairs / computed : 0.0;
    if (total_out) *total_out = total;
    if (stats_out) *stats_out = stats;
    return EJOIN_OK;
}

}  // namespace ejoin

using namespace ejoin;

extern "C" {

int ejoin_default_options(ejoin_options* opt) {
    if (!opt) return set_error(EJOIN_EINVAL, "opt is NULL");
    memset(opt, 0, sizeof *opt);
    opt->struct_size = sizeof(ejoin_options);
    opt->device = 0;
    opt->precision = EJOIN_AUTO;
    opt->proj_k = 0;
    opt->train_pairs = 1u << 19;
    opt->train_steps = 50;
    opt->order = EJOIN_ORDER_MORTON;
    opt->seed = 0x5eed5eedull;
    opt->acc_bound_scale = 1.0;
    return EJOIN_OK;
}

int ejoin_self_join(const double* points, uint64_t n, uint32_t d, double eps,
                    const ejoin_options* opt, int32_t* counts_out, uint64_t* total_out,
                    ejoin_stats* stats_out) {
    clear_error();
    NvtxRange nr("ejoin_self_join");
    return self_join_impl(points, n, d, eps, opt, counts_out, total_out, stats_out);
}

int ejoin_neighbor_lists(const double* points, uint64_t n, uint32_t d, double eps,
                         const ejoin_options* opt, uint64_t* offsets, uint32_t* neighbors,
                         uint64_t capacity, uint64_t* total_out, ejoin_stats* stats_out) {
    clear_error();
    if (!offsets) return set_error(EJOIN_EINVAL, "offsets is NULL");
    ListsReq req{offsets, neighbors, capacity};
    EJ_TRY(self_join_impl(points, n, d, eps, opt, nullptr, total_out, stats_out, &req));
    return req.status;
}

int ejoin_query_counts(const double* points, uint64_t n, uint32_t d, double eps,
                       const uint64_t* rows, uint64_t nq, const ejoin_options* opt_in,
                       int32_t* counts_out) {
    clear_error();
    ejoin_options opt;
    ejoin_default_options(&opt);
    if (opt_in) {
        if (opt_in->struct_size != sizeof(ejoin_options)) return set_error(EJOIN_EINVAL, "ejoin_options.struct_size mismatch");
        opt = *opt_in;
    }
    if (d == 0 || (n && !points) || (nq && (!rows || !counts_out)))
        return set_error(EJOIN_EINVAL, "bad arguments");
    const uint64_t ld = opt.ld ? opt.ld : d;
    if (ld < d) return set_error(EJOIN_EINVAL, "row stride < d");
    DeviceScope ds;
    int sms = 0;
    EJ_TRY(check_device(opt.device, &sms));
    EJ_TRY(ds.enter(opt.device));
    cudaStream_t s = opt.stream ? (cudaStream_t)opt.stream : cudaStreamPerThread;
    CallScope scope;  // before every device buffer of the call
    EJ_TRY(scope.enter(opt.device, s, (opt.flags & EJOIN_FLAG_KEEP_SCRATCH) != 0));
    const double T = threshold(eps);
    const bool out_dev = is_device_ptr(counts_out);
    DBuf<double> xbuf;
    const double* X = nullptr;
    DBuf<uint64_t> rbuf;
    DBuf<int32_t> cbuf;
    EJ_TRY(cbuf.alloc(nq ? nq : 1, s, "query counts"));
    EJ_TRY(cbuf.zero(s));
    if (n && nq && !isnan(T) && T >= 0.0) {
        EJ_TRY(stage_points(points, n, d, ld, xbuf, &X, s));
        for (uint64_t i = 0; i < nq; ++i) {
            if (!is_device_ptr(rows) && rows[i] >= n)
                return set_error(EJOIN_EINVAL, "query row %llu >= n", (unsigned long long)rows[i]);
        }
        EJ_TRY(rbuf.alloc(nq, s, "query rows"));
        EJ_CUDA(cudaMemcpyAsync(rbuf.p, rows, nq * sizeof(uint64_t), cudaMemcpyDefault, s));
        EJ_TRY(launch_direct_query(X, n, d, T, rbuf.p, nq, cbuf.p, s));
    }
    if (nq)
        EJ_CUDA(cudaMemcpyAsync(counts_out, cbuf.p, nq * sizeof(int32_t),
                                out_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    return EJOIN_OK;
}

// Join of two point sets on the tensor-core screen: queries are the A side
// (rows, counted), points the B side; both centred with the points' mean and
// packed with one scale.  Data outside the FP32 path's range, FP64 modes and
// eps = inf take the exact FP64 arbiter.
static int cross_join(Join& J, const double* Xq, uint64_t nq, int prec, int32_t* qcounts) {
    const bool fp64 = prec == EJOIN_FP64_DIRECT || prec == EJOIN_FP64_DMMA || isinf(J.T);
    if (!fp64) {
        const Fmt fmt = prec == EJOIN_FP16 ? Fmt::FP16 : (prec == EJOIN_FP8_E4M3 ? Fmt::E4M3 : Fmt::BF16);
        const bool split = prec == EJOIN_BF16_SPLIT;
        EventTimer tp, tg, tr;
        tp.start(J.s);
        DBuf<uint8_t> badx, badq;
        DBuf<double> mu;
        DBuf<float> Yx, Ex, Yq, Eq;
        EJ_TRY(badx.alloc(J.n, J.s, "row flags"));
        EJ_TRY(badq.alloc(nq, J.s, "query flags"));
        EJ_TRY(mu.alloc(J.d, J.s, "mean"));
        EJ_TRY(Yx.alloc(J.n * J.d, J.s, "FP32 centred points"));
        EJ_TRY(Ex.alloc(J.n, J.s, "centring error bounds"));
        EJ_TRY(Yq.alloc(nq * J.d, J.s, "FP32 centred queries"));
        EJ_TRY(Eq.alloc(nq, J.s, "centring error bounds"));
        CenterStats cx, cq;
        EJ_TRY(launch_center_stats(J.X, J.n, J.d, badx.p, mu.p, Yx.p, Ex.p, &cx, J.s));
        EJ_TRY(launch_center_stats(Xq, nq, J.d, badq.p, mu.p, Yq.p, Eq.p, &cq, J.s, true));
        const double maxabs = std::max(cx.maxy, cq.maxy);
        const bool flushed = cx.flushed || cq.flushed;
        const bool fp32_ok = !cx.range && !cq.range &&
                             (maxabs == 0.0 ? !flushed : (maxabs >= 0x1p-50 && maxabs <= 0x1p50));
        if (fp32_ok) {
            double kprod = 0;
            const ScreenParams P =
                screen_params(fmt, split, J.d, maxabs, J.T, J.opt.acc_bound_scale, &kprod);
            PackedSide sx, sq;
            const uint64_t npx = round_up(J.n, 256), npq = round_up(nq, 128);
            EJ_TRY(pack_side(Yx.p, Ex.p, badx.p, J.n, npx, nullptr, P, sx, J.s));
            EJ_TRY(pack_side(Yq.p, Eq.p, badq.p, nq, npq, nullptr, P, sq, J.s));
            tp.stop(J.s);
            J.st->ms_prep = tp.ms();
            DBuf<uint2> work;
            uint64_t nwork = 0, ntiles = 0;
            const uint64_t nTq = (nq + 127) / 128, nTx = (J.n + 127) / 128;
            EJ_TRY(build_worklist_cross(nTq, nTx, work, &nwork, &ntiles, J.s));
            J.st->tile_pairs_total = nTq * nTx;
            J.st->tile_pairs_run = ntiles;
            J.st->reserved[1] = (double)nwork;
            J.st->gram_flops = 2.0 * kprod * 128.0 * 256.0 * (double)nwork;
            J.st->precision = prec;
            Join Jq = J;  // counts of the screen: the queries (A side)
            Jq.counts = qcounts;
            const GramSide A{sq.operands(P), sq.Aug.p, npq}, B{sx.operands(P), sx.Aug.p, npx};
            auto screen = [&](BandPair* band, uint64_t cap, DevStatus* st) {
                return launch_gram16(A, B, P, work.p, nwork, sx.cmax.p, sq.beta.p, sx.tsig.p,
                                     sq.sig.p, true, qcounts, reinterpret_cast<BandRec*>(band), cap,
                                     st, nullptr, J.sms, J.s);
            };
            Recheck32 R;
            R.Xf = sq.Xf.p;
            R.rad = sq.rad.p;
            R.Xfb = sx.Xf.p;
            R.radb = sx.rad.p;
            if (sq.Xh.p && sx.Xh.p) {
                R.Xh = sq.Xh.p;
                R.radh = sq.radh.p;
                R.Xhb = sx.Xh.p;
                R.radhb = sx.radh.p;
            }
            R.Xb = J.X;
            R.nb = J.n;
            R.permb = nullptr;
            R.sTlo = P.sTlo;
            R.sThi = P.sThi;
            R.c32 = (J.d + 8) * ldexp(1.0, -24) * 1.01;
            R.abs32 = (J.d + 8) * ldexp(1.0, -148);
            finish_recheck32(R);
            auto recheck = [&](const BandPair* band, uint64_t nrec, uint64_t npairs, DevStatus* st) {
                if (npairs == 0) return EJOIN_OK;
                DBuf<BandPair> pairs;
                EJ_TRY(pairs.alloc(npairs, J.s, "band pairs"));
                EJ_TRY(launch_band_expand(reinterpret_cast<const BandRec*>(band), nrec, pairs.p,
                                          npairs, J.s));
                return launch_band_recheck2(Xq, nq, J.d, nullptr, J.T, R, pairs.p, npairs, qcounts,
                                            st, nullptr, J.s);
            };
            const uint64_t cap0 = std::max<uint64_t>(1u << 22, 16 * (nq + J.n));
            return screen_and_recheck(Jq, cap0, screen, recheck, npq, tg, tr, 2);
        }
    }
    EventTimer tg;
    tg.start(J.s);
    EJ_CUDA(cudaMemsetAsync(qcounts, 0, nq * sizeof(int32_t), J.s));
    EJ_TRY(launch_direct_query(J.X, J.n, J.d, J.T, nullptr, nq, qcounts, J.s, Xq));
    tg.stop(J.s);
    J.st->ms_gram = tg.ms();
    J.st->precision = EJOIN_FP64_DIRECT;
    J.st->gram_flops = 3.0 * J.d * (double)nq * (double)J.n;
    return EJOIN_OK;
}

int ejoin_join_counts(const double* queries, uint64_t nq, const double* points, uint64_t n,
                      uint32_t d, double eps, const ejoin_options* opt_in, int32_t* counts_out,
                      uint64_t* total_out, ejoin_stats* stats_out) {
    clear_error();
    ejoin_options opt;
    ejoin_default_options(&opt);
    if (opt_in) {
        if (opt_in->struct_size != sizeof(ejoin_options))
            return set_error(EJOIN_EINVAL, "ejoin_options.struct_size mismatch");
        opt = *opt_in;
    }
    if (d == 0 || (n && !points) || (nq && !queries)) return set_error(EJOIN_EINVAL, "bad arguments");
    if (n > 0x7fffff00ull || nq > 0x7fffff00ull)
        return set_error(EJOIN_EUNSUPPORTED, "point sets above 2^31 - 256 rows");
    if (opt.proj_k) return set_error(EJOIN_EUNSUPPORTED, "learned pruning is for self joins (proj_k must be 0)");
    if (opt.precision < EJOIN_FP64_DIRECT || opt.precision > EJOIN_AUTO)
        return set_error(EJOIN_EINVAL, "unknown precision mode %d", opt.precision);
    if (opt.acc_bound_scale < 1.0) return set_error(EJOIN_EINVAL, "acc_bound_scale must be >= 1");
    const uint64_t ld = opt.ld ? opt.ld : d;
    if (ld < d) return set_error(EJOIN_EINVAL, "row stride < d");
    ejoin_stats stats;
    memset(&stats, 0, sizeof stats);
    stats.n = n;
    stats.d = d;
    DeviceScope ds;
    int sms = 0;
    EJ_TRY(check_device(opt.device, &sms));
    EJ_TRY(ds.enter(opt.device));
    cudaStream_t s = opt.stream ? (cudaStream_t)opt.stream : cudaStreamPerThread;
    CallScope scope;  // before every device buffer of the call
    EJ_TRY(scope.enter(opt.device, s, (opt.flags & EJOIN_FLAG_KEEP_SCRATCH) != 0));
    const double T = threshold(eps);
    const uint64_t launches0 = launches_so_far();
    EventTimer tt;
    tt.start(s);
    Join J;
    J.s = s;
    J.sms = sms;
    J.n = n;
    J.d = d;
    J.eps = eps;
    J.T = T;
    J.opt = opt;
    J.st = &stats;
    J.perm = nullptr;
    DBuf<double> xbuf, qbuf;
    DBuf<int32_t> cbuf;
    const uint64_t npq = round_up(std::max<uint64_t>(nq, 1), 128);
    EJ_TRY(cbuf.alloc(npq, s, "query counts"));
    EJ_TRY(cbuf.zero(s));
    int prec = resolve_precision(opt.precision, d);
    stats.precision = prec;
    if (n > 0 && nq > 0 && !isnan(T) && T >= 0.0) {
        const double* Xq = nullptr;
        EJ_TRY(stage_points(points, n, d, ld, xbuf, &J.X, s));
        EJ_TRY(stage_points(queries, nq, d, ld, qbuf, &Xq, s));
        EJ_TRY(cross_join(J, Xq, nq, prec, cbuf.p));
    }
    DBuf<unsigned long long> tot;
    EJ_TRY(tot.alloc(1, s, "total"));
    EJ_TRY(tot.zero(s));
    EJ_TRY(sum_counts(cbuf.p, nq, tot.p, s));
    if (counts_out && nq)
        EJ_CUDA(cudaMemcpyAsync(counts_out, cbuf.p, nq * sizeof(int32_t),
                                is_device_ptr(counts_out) ? cudaMemcpyDeviceToDevice
                                                          : cudaMemcpyDeviceToHost, s));
    unsigned long long total = 0;
    EJ_CUDA(cudaMemcpyAsync(&total, tot.p, sizeof total, cudaMemcpyDeviceToHost, s));
    tt.stop(s);
    EJ_CUDA(cudaStreamSynchronize(s));
    stats.ms_total = tt.ms();
    stats.kernel_launches = launches_so_far() - launches0;
    stats.reserved[2] = (double)scope.peak_reserved();
    const double computed = (double)n * (double)nq;
    stats.band_fraction = computed > 0 ? (double)stats.band_pairs / computed : 0.0;
    if (total_out) *total_out = total;
    if (stats_out) *stats_out = stats;
    return EJOIN_OK;
}

int ejoin_train_projection(const double* points, uint64_t n, uint32_t d, double eps,
                           const ejoin_options* opt_in, float* P_out, double* sigma_cert_out,
                           ejoin_stats* stats_out) {
    clear_error();
    ejoin_options opt;
    ejoin_default_options(&opt);
    if (opt_in) {
        if (opt_in->struct_size != sizeof(ejoin_options)) return set_error(EJOIN_EINVAL, "ejoin_options.struct_size mismatch");
        opt = *opt_in;
    }
    if (d == 0 || n < 2 || !points || !P_out) return set_error(EJOIN_EINVAL, "bad arguments");
    if (opt.proj_k == 0 || opt.proj_k > 16) return set_error(EJOIN_EINVAL, "proj_k must be in 1..16");
    if (!(eps > 0.0) || isinf(eps)) return set_error(EJOIN_EINVAL, "eps must be positive and finite");
    const uint64_t ld = opt.ld ? opt.ld : d;
    if (ld < d) return set_error(EJOIN_EINVAL, "row stride < d");
    DeviceScope ds;
    int sms = 0;
    EJ_TRY(check_device(opt.device, &sms));
    EJ_TRY(ds.enter(opt.device));
    cudaStream_t s = opt.stream ? (cudaStream_t)opt.stream : cudaStreamPerThread;
    CallScope scope;  // before every device buffer of the call
    EJ_TRY(scope.enter(opt.device, s, (opt.flags & EJOIN_FLAG_KEEP_SCRATCH) != 0));
    DBuf<double> xbuf;
    const double* X = nullptr;
    EJ_TRY(stage_points(points, n, d, ld, xbuf, &X, s));
    EventTimer t;
    t.start(s);
    DBuf<uint8_t> bad;
    DBuf<double> mu;
    EJ_TRY(bad.alloc(n, s, "row flags"));
    EJ_TRY(mu.alloc(d, s, "mean"));
    DBuf<float> Y32;
    EJ_TRY(Y32.alloc(n * d, s, "FP32 centred points"));
    CenterStats cs;
    EJ_TRY(launch_center_stats(X, n, d, bad.p, mu.p, Y32.p, nullptr, &cs, s));
    TrainResult tr;
    EJ_TRY(train_projection_dev(Y32.p, bad.p, training_rows(n), d, eps, opt.proj_k,
                                opt.train_pairs, opt.train_steps, opt.seed,
                                opt.order == EJOIN_ORDER_LEAD, s, tr));
    t.stop(s);
    memcpy(P_out, tr.P.data(), tr.P.size() * sizeof(float));
    if (sigma_cert_out) *sigma_cert_out = tr.sigma_cert;
    if (stats_out) {
        memset(stats_out, 0, sizeof *stats_out);
        stats_out->n = n;
        stats_out->d = d;
        stats_out->sigma_cert = tr.sigma_cert;
        stats_out->ms_train = t.ms();
        stats_out->reserved[0] = tr.loss_first;
        stats_out->reserved[1] = tr.loss_last;
    }
    return EJOIN_OK;
}

int ejoin_release_scratch(int device) {
    clear_error();
    if (device < 0 || device >= kMaxDevices) return set_error(EJOIN_EINVAL, "device %d out of range", device);
    cudaMemPool_t p = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        p = g_pools[device];
    }
    if (p) EJ_CUDA(cudaMemPoolTrimTo(p, 0));
    return EJOIN_OK;
}

int ejoin_testing_inject(int what, uint64_t value) {
    clear_error();
    switch (what) {
        case EJOIN_TESTING_FAIL_ALLOC: inject_alloc_failure(value); return EJOIN_OK;
        case EJOIN_TESTING_GRAM_TIMEOUT: inject_gram_timeout(value); return EJOIN_OK;
        default: return set_error(EJOIN_EINVAL, "unknown injection %d", what);
    }
}

double ejoin_threshold(double eps) { return threshold(eps); }

int ejoin_last_error(char* buf, size_t len) {
    if (buf && len) {
        strncpy(buf, t_msg, len - 1);
        buf[len - 1] = 0;
    }
    return t_status;
}

int ejoin_version(void) { return EJOIN_VERSION_MAJOR * 100 + EJOIN_VERSION_MINOR; }

void ejoin_free(void* p) { host_free(p); }

int ejoin_gpu_join_main_brute_force(unsigned int searchMode, unsigned int device, double* dataset,
                                    unsigned int* nbQueryPoints, double* epsilon,
                                    uint64_t* totalNeighbors, unsigned int input_dim,
                                    unsigned int compute_dim) {
    clear_error();
    if (!nbQueryPoints || !epsilon || !totalNeighbors)
        return set_error(EJOIN_EINVAL, "NULL argument");
    if (input_dim == 0 || compute_dim < input_dim)
        return set_error(EJOIN_EINVAL, "bad dimensions (input %u, compute %u)", input_dim, compute_dim);
    ejoin_options opt;
    ejoin_default_options(&opt);
    opt.device = (int32_t)device;
    opt.ld = compute_dim;
    switch (searchMode) {
        case 1: case 2: opt.precision = EJOIN_FP64_DIRECT; break;  // SM_GPU, SM_CUDA_ALT
        case 3: case 4: opt.precision = EJOIN_AUTO; break;         // SM_TENSOR, SM_TENSOR_MQ
        case 5: opt.precision = EJOIN_AUTO; opt.proj_k = 8; break; // learned pruning
        default: return set_error(EJOIN_EINVAL, "Unknown search mode %u", searchMode);
    }
    uint64_t total = 0;
    int rc = self_join_impl(dataset, *nbQueryPoints, input_dim, *epsilon, &opt, nullptr, &total, nullptr);
    if (rc == EJOIN_OK) *totalNeighbors = total;
    return rc;
}

}  // extern "C"
