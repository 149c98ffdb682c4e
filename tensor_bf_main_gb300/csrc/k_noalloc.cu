// k_noalloc.cu -- the exact join for callers that cannot allocate device memory.
//
// Some hosts of this join cannot call cudaMalloc while they run it: a
// database or stream engine that owns every byte of device memory through its
// own pool, a latency-critical service that forbids allocation (and the
// implicit synchronisation it brings) on its serving path, or a process
// sharing the GPU under a hard memory cap.  For them ejoin_self_join_noalloc
// runs the plain FP64 tensor-core join (the DMMA Gram screen of k_dmma.cu plus
// the FP64 band recheck of k_direct.cu, so the counts are exact) with every
// byte of scratch -- row flags, mean, centred rows, per-row thresholds, the
// band queue, the status word and the total -- carved from one file-scope
// static device array.  The caller passes device-resident points and counts.
//
// Limits and rules (also in include/ejoin.h):
//  * n <= 16384 and d <= 128 (the centred FP64 rows fill half of the array);
//    larger inputs are rejected with EJOIN_EINVAL before anything runs, and a
//    band larger than the queue's share of the array fails with EJOIN_ENOMEM;
//  * the array (32 MiB) is held by every GPU that loads the library until the
//    process exits;
//  * the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (the host-side name is only a stand-in); make that
//    first call before any stream capture on that device;
//  * points and counts must be memory of that device (or managed memory);
//    anything else is rejected with EJOIN_EINVAL before any launch;
//  * every call waits for its own work on `stream` before it returns (it
//    reads the status and the total back to the host);
//  * on a non-zero return the counts are zero, not partial sums;
//  * all calls share the one array: calls whose work overlaps on the GPU (two
//    streams, two threads) race and corrupt each other's results.  Each call
//    clears what must start at zero (status, counts, total).
#include <mutex>

#include "ejoin_internal.cuh"

namespace ejoin {

void oracle_band(double T, uint32_t d, double* Tlo, double* Thi);
double threshold(double eps);

namespace {

constexpr uint64_t kMaxN = 16384;
constexpr uint32_t kMaxD = 128;
constexpr size_t kScratchBytes = 32ull << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_addr[64] = {};

// Device address of the scratch array for the current device `dev`.
int scratch_address(int dev, unsigned char** out) {
    if (dev < 0 || dev >= 64) return set_error(EJOIN_EINVAL, "device ordinal %d unsupported", dev);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return cuda_error(e, "cudaGetSymbolAddress(scratch)", __FILE__, __LINE__);
        g_scratch_addr[dev] = p;
    }
    *out = (unsigned char*)g_scratch_addr[dev];
    return EJOIN_OK;
}

__global__ void na_rowflags_kernel(const double* __restrict__ X, uint64_t n, uint32_t d,
                                   uint8_t* bad) {
    const uint64_t row = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    bool ok = true;
    if (row < n)
        for (uint32_t k = lane; k < d; k += 32) ok &= isfinite(X[row * d + k]) != 0;
    ok = __all_sync(0xffffffffu, ok);
    if (row < n && lane == 0) bad[row] = ok ? 0 : 1;
}

// Mean over the finite rows, one block per 32 columns: warp w sums rows w,
// w + 32, w + 64, ... of its 32 columns (lane = column, coalesced 256-byte
// rows), then the 32 partial sums of each column are added in a fixed tree
// order, so the mean is the same on every run.
constexpr int kMeanWarps = 32;
__global__ void __launch_bounds__(kMeanWarps * 32)
    na_mean_kernel(const double* __restrict__ X, uint64_t n, uint32_t d,
                   const uint8_t* __restrict__ bad, double* mu) {
    __shared__ double part[kMeanWarps][33];
    __shared__ uint32_t good[kMeanWarps];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t k = blockIdx.x * 32u + lane;
    double s = 0.0;
    uint32_t g = 0;
    for (uint64_t r = w; r < n; r += kMeanWarps) {
        if (bad[r]) continue;
        ++g;
        if (k < d) s += X[r * d + k];
    }
    part[w][lane] = s;
    if (lane == 0) good[w] = g;
    __syncthreads();
    for (int h = kMeanWarps / 2; h > 0; h >>= 1) {
        if ((int)w < h) {
            part[w][lane] += part[w + h][lane];
            if (lane == 0) good[w] += good[w + h];
        }
        __syncthreads();
    }
    if (w == 0 && k < d) mu[k] = good[0] ? part[0][lane] / (double)good[0] : 0.0;
}

// Memory the kernels on `dev` can read and write without peer access:
// device memory of `dev` itself, or managed memory.
bool is_device_pointer(const void* p, int dev) {
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice && a.device == dev) || a.type == cudaMemoryTypeManaged;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

int run(const double* X, uint64_t n, uint32_t d, double eps, cudaStream_t s, int dev,
        int32_t* counts, uint64_t* total_out) {
    unsigned char* base = nullptr;
    EJ_TRY(scratch_address(dev, &base));
    const uint64_t n_pad = (n + 63) / 64 * 64;
    DmmaParams P;
    P.d = d;
    P.dp = (d + 31) / 32 * 32;
    const double T = threshold(eps);
    oracle_band(T, d, &P.Tlo, &P.Thi);
    P.sTlo = sqrt(P.Tlo) * (1 - 4 * kU);
    P.sThi = sqrt(P.Thi) * (1 + 4 * kU);
    P.crel = 2.0 * (P.dp + 8) * kU;

    size_t off = 0;
    auto carve = [&](size_t bytes) {
        unsigned char* p = base + off;
        off = align256(off + bytes);
        return p;
    };
    DevStatus* st = (DevStatus*)carve(sizeof(DevStatus));
    unsigned long long* tot = (unsigned long long*)carve(sizeof(unsigned long long));
    uint8_t* bad = carve(n_pad);
    double* mu = (double*)carve(sizeof(double) * P.dp);
    double* Y = (double*)carve(sizeof(double) * n_pad * P.dp);
    double* h = (double*)carve(sizeof(double) * n_pad);
    double* g = (double*)carve(sizeof(double) * n_pad);
    if (off >= kScratchBytes) return set_error(EJOIN_EINTERNAL, "scratch layout exceeds the array");
    BandPair* band = (BandPair*)(base + off);
    const uint64_t cap = (kScratchBytes - off) / sizeof(BandPair);

    EJ_CUDA(cudaMemsetAsync(st, 0, sizeof(DevStatus), s));
    EJ_CUDA(cudaMemsetAsync(tot, 0, sizeof(unsigned long long), s));
    if (n) EJ_CUDA(cudaMemsetAsync(counts, 0, n * sizeof(int32_t), s));
    if (n == 0 || isnan(T) || T < 0.0) {
        unsigned long long zero = 0;
        if (total_out) *total_out = zero;
        EJ_CUDA(cudaStreamSynchronize(s));
        return EJOIN_OK;
    }
    if (isinf(T)) {
        // every non-NaN pair counts: the exact direct arbiter needs no scratch
        EJ_TRY(launch_direct_selfjoin(X, n, d, T, counts, nullptr, s));
    } else {
        na_rowflags_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(X, n, d, bad);
        EJ_CUDA(cudaGetLastError());
        note_launch();
        na_mean_kernel<<<(d + 31) / 32, kMeanWarps * 32, 0, s>>>(X, n, d, bad, mu);
        EJ_CUDA(cudaGetLastError());
        note_launch();
        EJ_TRY(launch_pack_dmma(X, n, n_pad, nullptr, bad, mu, P, Y, h, g, s));
        EJ_TRY(launch_dmma_join(Y, n_pad, P.dp, h, g, counts, band, cap, st, s));
        DevStatus hs;
        EJ_CUDA(cudaMemcpyAsync(&hs, st, sizeof hs, cudaMemcpyDeviceToHost, s));
        EJ_CUDA(cudaStreamSynchronize(s));
        // on either failure the screen's partial counts are cleared, so a
        // caller that ignores the status reads zeros, not plausible counts
        if (hs.timeout) {
            EJ_CUDA(cudaMemsetAsync(counts, 0, n * sizeof(int32_t), s));
            EJ_CUDA(cudaStreamSynchronize(s));
            return set_error(EJOIN_ETIMEOUT, "a bounded device wait expired");
        }
        if (hs.band_count > cap) {
            EJ_CUDA(cudaMemsetAsync(counts, 0, n * sizeof(int32_t), s));
            EJ_CUDA(cudaStreamSynchronize(s));
            return set_error(EJOIN_ENOMEM,
                             "boundary band of %llu pairs exceeds the %llu-entry queue of the "
                             "static scratch; use ejoin_self_join",
                             (unsigned long long)hs.band_count, (unsigned long long)cap);
        }
        EJ_TRY(launch_band_recheck(X, n, d, nullptr, T, band, hs.band_count, counts, st, s));
    }
    EJ_TRY(sum_counts(counts, n, tot, s));
    unsigned long long t = 0;
    EJ_CUDA(cudaMemcpyAsync(&t, tot, sizeof t, cudaMemcpyDeviceToHost, s));
    EJ_CUDA(cudaStreamSynchronize(s));
    if (total_out) *total_out = t;
    return EJOIN_OK;
}

}  // namespace
}  // namespace ejoin

using namespace ejoin;

extern "C" int ejoin_self_join_noalloc(const double* points, uint64_t n, uint32_t d, double eps,
                                       int device, void* stream, int32_t* counts,
                                       uint64_t* total_out) {
    clear_error();
    if (d == 0 || d > kMaxD)
        return set_error(EJOIN_EINVAL, "ejoin_self_join_noalloc: d = %u outside 1..%u", d, kMaxD);
    if (n > kMaxN)
        return set_error(EJOIN_EINVAL, "ejoin_self_join_noalloc: n = %llu exceeds the limit %llu",
                         (unsigned long long)n, (unsigned long long)kMaxN);
    if (n && (!points || !counts))
        return set_error(EJOIN_EINVAL, "ejoin_self_join_noalloc: NULL points or counts");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return set_error(EJOIN_ENODEV, "no CUDA device available");
    }
    if (device < 0 || device >= count) return set_error(EJOIN_EINVAL, "device %d out of range", device);
    cudaDeviceProp p;
    EJ_CUDA(cudaGetDeviceProperties(&p, device));
    if (p.major != 10 || p.minor != 3)
        return set_error(EJOIN_ENODEV, "device %d is sm_%d%d; the library is built for sm_103a", device,
                         p.major, p.minor);
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) {
        cudaGetLastError();
        prev = -1;
    }
    EJ_CUDA(cudaSetDevice(device));
    int rc = EJOIN_OK;
    if (n && (!is_device_pointer(points, device) || !is_device_pointer(counts, device)))
        rc = set_error(EJOIN_EINVAL,
                       "ejoin_self_join_noalloc: points and counts must be device memory of "
                       "device %d", device);
    else
        rc = run(points, n, d, eps, stream ? (cudaStream_t)stream : cudaStreamPerThread, device,
                 counts, total_out);
    if (prev >= 0) cudaSetDevice(prev);
    return rc;
}
