// ejoin_internal.cuh -- definitions shared by the translation units of
// libejoin.so.  Host: status/error plumbing, stream-ordered device buffers,
// event timers.  Device: the exact FP64 pair arithmetic of the reference
// (kernel_join.cu:184-199) and the band-queue record.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <functional>
#include <string>
#include <vector>

#include "ejoin.h"

namespace ejoin {

// ---------------------------------------------------------------- errors --

int set_error(int status, const char* fmt, ...);
// Kernel launches issued by the calling thread (reported in ejoin_stats).
void note_launch(uint64_t k = 1);
uint64_t launches_so_far();
int cuda_error(cudaError_t e, const char* what, const char* file, int line);
void clear_error();

#define EJ_CUDA(expr)                                                        \
    do {                                                                     \
        cudaError_t _e = (expr);                                             \
        if (_e != cudaSuccess) return ::ejoin::cuda_error(_e, #expr, __FILE__, __LINE__); \
    } while (0)

#define EJ_TRY(expr)                  \
    do {                              \
        int _rc = (expr);             \
        if (_rc != EJOIN_OK) return _rc; \
    } while (0)

// ------------------------------------------------------- device buffers --

// Device scratch comes from a memory pool the library owns, one per device
// (never the device's default pool, which belongs to the host program).
// CallScope, constructed by every entry point before its first buffer,
// selects the pool for the calling thread; when the entry point returns (its
// buffers freed, its stream synchronised) the pool gives its memory back to
// the device unless the caller asked to keep it (EJOIN_FLAG_KEEP_SCRATCH).
cudaMemPool_t current_pool();
struct CallScope {
    cudaMemPool_t pool = nullptr, prev = nullptr;
    cudaStream_t s = nullptr;
    bool keep = false;
    // Selects the library pool of device dev for this thread (creating it
    // on first use).
    int enter(int dev, cudaStream_t stream, bool keep_scratch);
    // Largest device memory the pool reserved since enter() (bytes).
    uint64_t peak_reserved() const;
    ~CallScope();
};
// Host result buffers of the loaders: page-locked where a CUDA device is
// present (else malloc); host_free releases either kind.
void* host_alloc(size_t bytes);
void host_free(void* p);

// Test hook: make the k-th device allocation from now fail (0 = none).
void inject_alloc_failure(uint64_t k);
bool alloc_should_fail();

// Stream-ordered device allocation from the library pool of the current
// call (freed blocks stay cached in the pool for the rest of the call).
// Freed on the same stream when the buffer goes out of scope.
template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t count = 0;
    cudaStream_t s = nullptr;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        count = 0;
    }
    int alloc(size_t n, cudaStream_t stream, const char* what) {
        release();
        s = stream;
        count = n;
        if (n == 0) return EJOIN_OK;
        cudaMemPool_t pool = current_pool();
        cudaError_t e = alloc_should_fail()
                            ? cudaErrorMemoryAllocation
                            : (pool ? cudaMallocFromPoolAsync((void**)&p, n * sizeof(T), pool, stream)
                                    : cudaMallocAsync((void**)&p, n * sizeof(T), stream));
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            return set_error(EJOIN_ENOMEM, "device allocation of %zu bytes for %s failed: %s",
                             n * sizeof(T), what, cudaGetErrorString(e));
        }
        return EJOIN_OK;
    }
    int zero(cudaStream_t stream) {
        if (!p) return EJOIN_OK;
        EJ_CUDA(cudaMemsetAsync(p, 0, count * sizeof(T), stream));
        return EJOIN_OK;
    }
};

struct EventTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    EventTimer() {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~EventTimer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    void start(cudaStream_t s) { cudaEventRecord(a, s); }
    void stop(cudaStream_t s) { cudaEventRecord(b, s); }
    double ms() {
        float v = 0.f;
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&v, a, b);
        return v;
    }
};

// ------------------------------------------------------------ constants --

constexpr double kU = 1.1102230246251565e-16;  // 2^-53, FP64 unit roundoff
constexpr double kTwo100 = 1.2676506002282294e30;  // 2^100

// Band-queue record: directed pair (i, j) in packed-row index space.  Bit 31
// of j is set when the pair also credits j (an off-diagonal tile pair: the
// tile kernels visit only I <= J, so (j, i) is never visited on its own).
struct BandPair {
    uint32_t i;
    uint32_t j;
};
constexpr uint32_t kBandBoth = 0x80000000u;

// Band record of the tensor-core screen: the pairs (i, j0 + c) for every set
// bit c of mask (j0 carries kBandBoth like BandPair::j).  One record per row
// of a 32 x 32 chunk with band pairs: the screen's epilogue writes a row's
// bit mask instead of expanding it (launch_band_expand does that later).
struct BandRec {
    uint32_t i;
    uint32_t j0;
    uint32_t mask;
    uint32_t pad;
};

// Pair emission for neighbour lists (null when only counts are wanted):
// in-records of the tensor-core screen and single pairs (band hits, direct
// arbiter hits), appended through the counters cnt[0] / cnt[1]; entries beyond
// a capacity are dropped and detected by the caller from the counters.
struct Emit {
    BandRec* inq;
    uint64_t inq_cap;
    BandPair* pq;
    uint64_t pq_cap;
    unsigned long long* cnt;  // [0] in-records, [1] pairs
};

// Kernels take an Emit by value; cnt == null means no emission.
__device__ __forceinline__ void emit_pair(const Emit& em, BandPair bp) {
    if (!em.cnt) return;
    const unsigned long long slot = atomicAdd(&em.cnt[1], 1ull);
    if (slot < em.pq_cap) em.pq[slot] = bp;
}

// Status word written by kernels whose waits are bounded.
struct DevStatus {
    unsigned int timeout;    // a bounded wait expired (where: code below)
    unsigned int where;
    unsigned long long band_count;  // band queue entries produced (may exceed capacity)
    unsigned long long band_pairs;  // pairs in those entries (record queues)
    unsigned long long band_hits;
    unsigned long long exact_rechecks;  // band pairs the FP32 pre-check left to FP64
    // test hooks (zero in normal runs): the deadline of the bounded waits in
    // ns (0 = the default), and, in the tensor-core Gram kernel, a producer
    // that never issues the copies of its first stage
    unsigned long long wait_ns;
    unsigned int withhold;
    unsigned int pad_;
    // record queues: records actually produced (band_count counts the queue
    // space reserved, which may include empty records, mask 0)
    unsigned long long band_records;
};
// Test hook: the next tensor-core screen runs with wait deadline `ns` and a
// producer that withholds its first stage (the waits then expire).
void inject_gram_timeout(uint64_t ns);
uint64_t take_gram_timeout();

// Constants of the FP32 band pre-check (scaled space of the 16-bit screen).
// Pairs (i, j) take row i from side A and row j from side B; for a self join
// the two sides are the same arrays.
struct Recheck32 {
    const float* Xf;   // A: [n_pad][d] FP32 coordinates, packed order
    const float* rad;  // A: per-row radius (|zf - s (x - mu)| bound; inf = undecidable row)
    const float* Xfb;  // B: the same for the second point set
    const float* radb;
    // optional first pass (wide bands of the FP8 screen): FP16 copies of the
    // coordinates with their own radius (rad + |zh - zf|); null = none
    const uint16_t* Xh = nullptr;
    const float* radh = nullptr;
    const uint16_t* Xhb = nullptr;
    const float* radhb = nullptr;
    const double* Xb;  // B: original FP64 rows (the exact chain)
    uint64_t nb;       // B: rows
    const uint32_t* permb;  // B: packed -> original row (null = identity)
    double sTlo, sThi; // sqrt of the scaled oracle thresholds (down / up)
    double c32;        // relative bound of the FP32 squared-difference sum
    double abs32;      // absolute bound (FP32 underflow)
    // the same constants as FP32 values rounded outward (finish_recheck32):
    // the per-pair decision runs in FP32 with directed rounding (FP64 is slow
    // on GB300)
    float f_sTlo, f_sThi;  // sTlo rounded down, sThi rounded up
    float f_kin, f_kout;   // 1 - c32 rounded down, 1 + c32 rounded up
    float f_abs;           // abs32 rounded up
};
// Fills the FP32 constants of R from its FP64 ones (host).
void finish_recheck32(Recheck32& R);

// --------------------------------------------------------- device math --

// Squared distance exactly as the reference's FP64 kernel computes it
// (kernel_join.cu:184-189 as nvcc compiles it for sm_103a): per coordinate
// t_k = a_k - b_k rounded once; the first two terms as fma(t0, t0, fl(t1*t1))
// (the compiler folds `0 + t0*t0` into the bare product and fuses that one
// into the second step), then acc = fma(t_k, t_k, acc) for k >= 2 in index
// order.  Running the reference's own compiled kernel on pairs built to tell
// the readings apart pinned this form at d = 18, 64 and 128.  d = 1 gives
// fl(t0*t0).
__device__ __forceinline__ double exact_d2(const double* __restrict__ a,
                                           const double* __restrict__ b, uint32_t d) {
    const double t0 = __dsub_rn(a[0], b[0]);
    const double t1 = d > 1 ? __dsub_rn(a[1], b[1]) : 0.0;
    double acc = __fma_rn(t0, t0, __dmul_rn(t1, t1));
    for (uint32_t k = 2; k < d; ++k) {
        const double t = __dsub_rn(a[k], b[k]);
        acc = __fma_rn(t, t, acc);
    }
    return acc;
}

// Decode linear index t of the row-major upper triangle of an nT x nT grid
// into (I, J), I <= J.
__device__ __forceinline__ void tri_decode(uint64_t t, uint64_t nT, uint64_t& I, uint64_t& J) {
    // row r holds nT - r entries and starts at r*nT - r*(r-1)/2
    double b = 2.0 * (double)nT + 1.0;
    double disc = b * b - 8.0 * (double)t;
    uint64_t i = (uint64_t)((b - sqrt(disc > 0 ? disc : 0.0)) * 0.5);
    if (i > nT - 1) i = nT - 1;
    auto first = [nT](uint64_t r) { return r * nT - r * (r - 1) / 2; };
    while (i > 0 && first(i) > t) --i;
    while (i + 1 < nT && first(i + 1) <= t) ++i;
    I = i;
    J = i + (t - first(i));
}

// Warp-aggregated append of `cnt` band pairs held by this lane; returns this
// lane's first slot (slots >= cap are dropped by the caller; the count still
// grows so the host can size a re-run).
__device__ __forceinline__ unsigned long long band_reserve(DevStatus* st, unsigned cnt) {
    const unsigned lane = threadIdx.x & 31;
    unsigned incl = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += v;
    }
    unsigned total = __shfl_sync(0xffffffffu, incl, 31);
    unsigned long long base = 0;
    if (lane == 31 && total) base = atomicAdd(&st->band_count, (unsigned long long)total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + (incl - cnt);
}

// ------------------------------------------------- screen parameters --

// Operand formats of the tensor-core screen.
enum class Fmt : int { BF16 = 0, FP16 = 1, E4M3 = 2 };

// Per-join constants of the screen's error bound (all in the scaled, centred
// coordinate space z = s * fl(x - mu) unless stated).
struct ScreenParams {
    double scale;      // s, a power of two
    double Tlo, Thi;   // s^2 * T_lo, s^2 * T_hi (oracle rounding folded in)
    double sTlo, sThi; // sqrt(Tlo) rounded down, sqrt(Thi) rounded up
    // tensor-core accumulation error of C_ij: |err| <= e_i + e_j with
    // 2 e_i = acc_margin2(a_i^2, l_i^2) + 2 cacc_al |alpha_i| (api.cu: screen_params)
    double cacc_a, cacc_l, cacc_al;
    double absacc;     // absolute bound (FP32 underflow) of the same
    double inv_in_pos; // 1 / (2 (1 - cacc_al)) rounded up
    double inv_in_neg; // 1 / (2 (1 + cacc_al)) rounded down
    double flush_err;  // 2^-126 sqrt(d) rounded up: coordinates flushed below FP32 range
    double clamp_lo;   // smallest alpha the operand format can carry
    uint32_t d, dp;    // coordinates, padded coordinates (per slab multiple)
    uint32_t width;    // packed row width in elements (dp, or 2 dp with the split)
    int split;         // 1 = hi + lo products
    Fmt fmt;
};

// The row's share of the accumulation bound that does not depend on alpha,
// doubled: cacc_a a^2 + cacc_l (2^-9 a^2 + 2^9 l^2), where a^2 bounds
// |(|hi| + |lo|)|^2 and l^2 bounds |lo|^2 (0 without the split).
__host__ __device__ __forceinline__ double acc_margin2(const ScreenParams& P, double a2, double l2) {
    return P.cacc_a * a2 + P.cacc_l * (a2 * (1.0 / 512.0) + l2 * 512.0);
}

// Per-join constants of the FP64 DMMA screen (unscaled centred space y).
struct DmmaParams {
    double Tlo, Thi, sTlo, sThi;
    double crel;       // relative bound (Gram + norms + epilogue rounding)
    uint32_t d, dp;
};

// Boxes of the projected 128-row tiles and of super-blocks of kSuperTiles
// consecutive tiles ([tiles][k] FP32, outward rounded).
constexpr uint32_t kSuperTiles = 16;
struct LearnedBoxes {
    DBuf<float> lo, hi, slo, shi;
    uint32_t k = 0;
};

// --------------------------------------------------- host entry points --
// (implemented in the kernel translation units)

struct JoinCtx;  // api.cu

// k_direct.cu
int launch_direct_selfjoin(const double* X, uint64_t n, uint32_t d, double T, int32_t* counts,
                           const Emit* em,
                           cudaStream_t s);
// Query counts against all n rows of X: query rows rows[q] of X, or (Xq
// non-null) the rows of a separate nq x d array Xq.
int launch_direct_query(const double* X, uint64_t n, uint32_t d, double T, const uint64_t* rows,
                        uint64_t nq, int32_t* counts, cudaStream_t s, const double* Xq = nullptr);
int launch_band_recheck(const double* X, uint64_t n, uint32_t d, const uint32_t* perm, double T,
                        const BandPair* band, uint64_t nband, int32_t* counts, DevStatus* st,
                        cudaStream_t s);

// k_dmma.cu: FP64 DMMA Gram screen over upper-triangle 64x64 tile pairs.
int launch_dmma_join(const double* Y, uint64_t n_pad, uint32_t dp, const double* h,
                     const double* g, int32_t* counts, BandPair* band, uint64_t band_cap,
                     DevStatus* st, cudaStream_t s);

// k_umma.cu: tcgen05 Gram screen over a tile-pair work list (16-bit operands).
// (FP8 operands: also the per-tile minimum row scale tsig.)
// One operand side of the tensor-core Gram screen: packed rows [n_pad][W]
// and aug rows [n_pad][32].
struct GramSide {
    const void* Q;
    const void* aug;
    uint64_t n_pad;
};
// Rows of A against columns of B over the blocks of the work list.  cmax_b:
// per 32-row chunk of B, max beta; beta_a: per row of A; FP8: tsig_b / sig_a
// per-tile minimum / per-row scales.  cross: A and B are different point
// sets (only A's rows are counted, every block as a diagonal one); else A is
// B and the upper-triangle blocks credit both sides.
int launch_gram16(const GramSide& A, const GramSide& B, const ScreenParams& P, const uint2* work,
                  uint64_t nwork, const float* cmax_b, const float* beta_a, const float* tsig_b,
                  const float* sig_a, bool cross, int32_t* counts, BandRec* band, uint64_t band_cap,
                  DevStatus* st, const Emit* em, int num_sms, cudaStream_t s);

// k_misc.cu
// Ordered list of 128 x 256 blocks (row tile I, column tiles Ja, Jb)
// covering the upper-triangle tile pairs (I <= J < nTa), grouped by
// super-block pairs; entry = (I | active-half mask << 30, Ja | (Jb - Ja) << 24);
// a row's active tiles within a super-block are paired.  With `boxes`,
// tile pairs whose squared box gap exceeds thr are inactive (super-block
// pairs are dropped first).  ntiles_out: active 128 x 128 tile pairs.
int build_worklist(uint64_t nT, uint64_t nTa, const LearnedBoxes* boxes, float thr,
                   DBuf<uint2>& work, uint64_t* nwork_out, uint64_t* ntiles_out, cudaStream_t s);
// All blocks of a join of two point sets: nTa row tiles (with data) against
// nTb column tiles (with data; B padded to whole 256-row pairs).
int build_worklist_cross(uint64_t nTa, uint64_t nTb, DBuf<uint2>& work, uint64_t* nwork_out,
                         uint64_t* ntiles_out, cudaStream_t s);
// out = work[0], work[stride], work[2 stride], ... (*nsample_out entries).
int sample_worklist(const uint2* work, uint64_t nwork, uint64_t stride, DBuf<uint2>& out,
                    uint64_t* nsample_out, cudaStream_t s);
int sum_counts(const int32_t* counts, uint64_t n, unsigned long long* dev_total, cudaStream_t s);
int scatter_counts(const int32_t* src, const uint32_t* perm, uint64_t n, int32_t* dst,
                   cudaStream_t s);

// k_learn.cu: learned projection, ordering, tile boxes
struct TrainResult {
    std::vector<float> P;
    double loss_first = 0, loss_last = 0;
    double sigma_cert = 0;
};
// Rows the projection training samples from: the first training_rows(n)
// rows (all rows up to 2^21, else half of them, at least 2^21), so that the
// training can start while the rest of a staged input is still copied.
inline uint64_t training_rows(uint64_t n) {
    return n <= (1ull << 21) ? n : std::max<uint64_t>(1ull << 21, n / 2);
}
// Y32: FP32 centred copy of the points (launch_center_stats); bad: row flags.
int train_projection_dev(const float* Y32, const uint8_t* bad, uint64_t n, uint32_t d, double eps,
                         uint32_t k, uint64_t pairs, uint32_t steps, uint64_t seed, int lead_only,
                         cudaStream_t s, TrainResult& out);
// Yerr (centring error bounds) is required with boxes: the boxes are rigorous.
// pmax >= max_a ||P_a||_2 (rounded up).
int learned_order(const float* Y32, const float* Yerr, const uint8_t* bad, uint64_t n,
                  uint64_t n_pad, uint32_t d, const float* P_dev, uint32_t k, float pmax,
                  int lead_only, DBuf<uint32_t>& perm, LearnedBoxes* boxes, cudaStream_t s);
// host.cpp: certified upper bound of ||P||_2
int cert_spectral_norm(const float* P, uint32_t k, uint32_t d, double* out);

// Expands band records into pairs (any order); out holds Sum popc(mask).
int launch_band_expand(const BandRec* rec, uint64_t nrec, BandPair* out, uint64_t cap,
                       cudaStream_t s);
// k_lists.cu: CSR neighbour lists.  offsets [n + 1] from the per-point counts
// (input order); csr_fill scatters the emitted pairs (packed indices, perm:
// packed -> input row) into nb [total] and sorts every list.
int csr_offsets(const int32_t* counts, uint64_t n, uint64_t total, unsigned long long* offsets,
                cudaStream_t s);
int csr_fill(const unsigned long long* offsets, uint64_t n, uint64_t total, const BandRec* inq,
             uint64_t nin, const BandPair* pq, uint64_t np, const uint32_t* perm, uint32_t* nb,
             cudaStream_t s);

int launch_band_recheck2(const double* X, uint64_t n, uint32_t d, const uint32_t* perm, double T,
                         const Recheck32& R, const BandPair* band, uint64_t nband, int32_t* counts,
                         DevStatus* st, const Emit* em, cudaStream_t s);

// k_prep.cu
// Centring statistics.  bad[i] = 1 for rows with a non-finite coordinate;
// mu = an FP32-representable mean (of a fixed sample of rows); with Y32 the
// FP32 centred copy [n][d] and Yerr[i] >= ||Y32_i - (x_i - mu)||_2.
struct CenterStats {
    double maxy = 0;       // max |Y32| over the finite rows
    uint64_t ngood = 0;    // finite rows
    bool range = false;    // a coordinate beyond 2^120: the FP32 copy is unusable
    bool flushed = false;  // a nonzero coordinate below 2^-126 was replaced by 0
};
// A host-to-device copy of the points left to the centring pass: X (device,
// allocated on the caller's stream) is filled from pinned host rows in
// chunks on a side stream, and each chunk is centred as soon as it lands, so
// the copy (bound by the host link) hides the centring.  host_dev is the
// device-side address of the same pinned rows (the sample for the mean is
// read from there before the copy completes).
struct StageCopy {
    const double* host;
    const double* host_dev;
};
// mu_given: mu holds the mean to use (another point set's, FP32-representable).
// sc: X is still to be copied from pinned host memory (null: X is in place).
// on_prefix (optional) is called once every copy and centring pass is
// enqueued, with an event on s that completes when the first prefix_rows rows
// are centred; it may run work on its own stream that waits for that event
// (the projection training), overlapping the rest of the copy.
using PrefixHook = std::function<int(cudaEvent_t)>;
int launch_center_stats(const double* X, uint64_t n, uint32_t d, uint8_t* bad, double* mu,
                        float* Y32, float* Yerr, CenterStats* out, cudaStream_t s,
                        bool mu_given = false, const StageCopy* sc = nullptr,
                        uint64_t prefix_rows = 0, const PrefixHook* on_prefix = nullptr);
// FP64 centred copy Y[n_pad][dp] and per-row thresholds h, g for the DMMA screen.
int launch_pack_dmma(const double* X, uint64_t n, uint64_t n_pad, const uint32_t* perm,
                     const uint8_t* bad, const double* mu, const DmmaParams& P, double* Y,
                     double* h, double* g, cudaStream_t s);
// 16-bit operand rows [hi | lo], aug rows [augA(16) | augB(16)], per-row
// out-margins beta, FP32 coordinates Xf ([n_pad][d], scaled, centred) and
// their per-row error radius.
int launch_pack16(const float* Y32, const float* Yerr, uint64_t n, uint64_t n_pad,
                  const uint32_t* perm, const uint8_t* bad, const ScreenParams& P, void* Q,
                  void* Aug, float* beta, float* Xf, float* rad, cudaStream_t s);
// E4M3 operand rows with per-row power-of-two scales sigma, BF16 aug rows,
// beta, sigma, FP32 coordinates / radii, and the per-tile minimum sigma.
int launch_pack8(const float* Y32, const float* Yerr, uint64_t n, uint64_t n_pad,
                 const uint32_t* perm, const uint8_t* bad, const ScreenParams& P, uint8_t* Q,
                 void* Aug, float* beta, float* sig, float* Xf, float* rad, float* tsig,
                 uint16_t* Xh, float* radh, cudaStream_t s);
// per group of 32 rows: max of beta (the band width of a 32-column chunk)
int launch_chunk_max(const float* beta, uint64_t n_pad, float* cmax, cudaStream_t s);

}  // namespace ejoin
