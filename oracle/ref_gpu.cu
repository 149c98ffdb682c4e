// ref_gpu.cu -- runs the reference's own join kernels on this GPU.
// TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the kernels come from
// oracle/_ref/ref_<variant>.cubin, compiled from the reference's
// kernel_join.cu by oracle/build_ref.sh; this program only loads them with the
// driver API and launches them the way the reference driver
// GPUJoinMainBruteForce does (gpu_join.cu:210-322):
//
//   dataset   (N + 15) rows x COMPUTE_DIM doubles, zero padded (main.cu:38-57,
//             ADDITIONAL_POINTS = 15, params.h:20)
//   cuda      searchMode 1 (SM_GPU): distanceCalculationBruteForceCuda
//             <<<ceil(N / 256), 256>>>(N, dataset, eps, cnt)  (gpu_join.cu:273-282)
//   mq16      searchMode 4, COMPUTE_PREC 16: convertDataset and
//             preComputedSquaredCoordinates <<<ceil((N + 15) / 256), 256>>>
//             over N + 15 rows (gpu_join.cu:224-255), then
//             distanceCalculationBruteForceTensorHalf
//             <<<ceil(2 N / 128), 128>>>(N, half data, float eps, cnt, norms)
//             (gpu_join.cu:301-304)
//   mq64      searchMode 4, COMPUTE_PREC 64: preComputedSquaredCoordinates
//             over N + 15 rows, then distanceCalculationBruteForceTensorDouble
//             <<<ceil(4 N / 128), 128>>>(N, data, double eps, cnt, norms)
//             (gpu_join.cu:305-307)
//
// Unlike the reference the counter is zeroed before every launch (it never
// was, gpu_join.cu:261-263), so the printed totals are what one launch
// counted.  Every kernel reads rows < N + 15 only (the candidate blocks of 16
// or 8 rows start below N), inside the padded buffer.
//
//   ref_gpu_launch <cubin> <cuda|mq16|mq64> <points.f64> <n> <input_dim>
//                  <compute_dim> <eps> [reps]
//
// prints one JSON line: the total, the join kernel's time per launch (CUDA
// events) and the time of the reference driver's whole sequence per run
// (allocation, host-to-device copy, conversion, norms, join, read-back: the
// window main.cu:60-110 times), best and mean over `reps` runs after one
// warm-up run.
#include <cuda.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <string>
#include <vector>

#define CK(x)                                                                        \
    do {                                                                             \
        CUresult _r = (x);                                                           \
        if (_r != CUDA_SUCCESS) {                                                    \
            const char* _s = nullptr;                                                \
            cuGetErrorString(_r, &_s);                                               \
            fprintf(stderr, "%s failed: %s (line %d)\n", #x, _s ? _s : "?", __LINE__); \
            exit(2);                                                                 \
        }                                                                            \
    } while (0)

static CUfunction find_kernel(CUmodule mod, const char* ident) {
    unsigned count = 0;
    CK(cuModuleGetFunctionCount(&count, mod));
    std::vector<CUfunction> fs(count);
    CK(cuModuleEnumerateFunctions(fs.data(), count, mod));
    for (CUfunction f : fs) {
        const char* name = nullptr;
        CK(cuFuncGetName(&name, f));
        // mangled name: _Z<len><identifier><parameters>
        const std::string want = std::to_string(strlen(ident)) + ident;
        if (name && strstr(name, want.c_str())) return f;
    }
    fprintf(stderr, "kernel %s not in the module\n", ident);
    exit(2);
}

static unsigned ceil_div(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }

int main(int argc, char** argv) {
    if (argc < 8) {
        fprintf(stderr, "usage: %s <cubin> <cuda|mq16|mq64> <points.f64> <n> <input_dim> "
                        "<compute_dim> <eps> [reps]\n", argv[0]);
        return 2;
    }
    const char* cubin = argv[1];
    const std::string kind = argv[2];
    const char* path = argv[3];
    const unsigned n = (unsigned)strtoul(argv[4], nullptr, 10);
    const unsigned din = (unsigned)strtoul(argv[5], nullptr, 10);
    const unsigned dc = (unsigned)strtoul(argv[6], nullptr, 10);
    const double eps = strtod(argv[7], nullptr);
    const int reps = argc > 8 ? atoi(argv[8]) : 1;
    if (kind != "cuda" && kind != "mq16" && kind != "mq64") return 2;
    if (n == 0 || din == 0 || dc < din || (kind == "mq16" && dc % 16) || (kind == "mq64" && dc % 4)) {
        fprintf(stderr, "bad sizes\n");
        return 2;
    }
    // points: n x din doubles, row-major
    std::vector<double> rows((size_t)n * din);
    FILE* f = fopen(path, "rb");
    if (!f || fread(rows.data(), sizeof(double), rows.size(), f) != rows.size()) {
        fprintf(stderr, "cannot read %s\n", path);
        return 2;
    }
    fclose(f);
    const size_t npad = (size_t)n + 15;
    std::vector<double> host(npad * dc, 0.0);
    for (size_t i = 0; i < n; ++i)
        memcpy(&host[i * dc], &rows[i * din], din * sizeof(double));

    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CUmodule mod;
    CK(cuModuleLoad(&mod, cubin));
    CUfunction kjoin, kconv = nullptr, knorm = nullptr;
    if (kind == "cuda") {
        kjoin = find_kernel(mod, "distanceCalculationBruteForceCuda");
    } else if (kind == "mq16") {
        kconv = find_kernel(mod, "convertDataset");
        knorm = find_kernel(mod, "preComputedSquaredCoordinates");
        kjoin = find_kernel(mod, "distanceCalculationBruteForceTensorHalf");
    } else {
        knorm = find_kernel(mod, "preComputedSquaredCoordinates");
        kjoin = find_kernel(mod, "distanceCalculationBruteForceTensorDouble");
    }
    CUevent e0, e1;
    CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    std::vector<double> kms, dms;
    unsigned long long total = 0;
    for (int r = 0; r <= reps; ++r) {
        const auto t0 = std::chrono::steady_clock::now();
        CUdeviceptr d_data, d_alt = 0, d_norm = 0, d_n, d_cnt, d_eps;
        CK(cuMemAlloc(&d_data, host.size() * sizeof(double)));
        CK(cuMemcpyHtoD(d_data, host.data(), host.size() * sizeof(double)));
        unsigned nb_tmp = ceil_div(npad, 256);
        unsigned npad_u = (unsigned)npad;
        if (kind == "mq16") {
            CK(cuMemAlloc(&d_alt, npad * dc * sizeof(__half)));
            void* ca[] = {&d_data, &d_alt, &npad_u};
            CK(cuLaunchKernel(kconv, nb_tmp, 1, 1, 256, 1, 1, 0, 0, ca, nullptr));
            CK(cuMemAlloc(&d_norm, npad * (dc / 16) * sizeof(float)));
            void* na[] = {&d_alt, &d_norm, &npad_u};
            CK(cuLaunchKernel(knorm, nb_tmp, 1, 1, 256, 1, 1, 0, 0, na, nullptr));
        } else if (kind == "mq64") {
            CK(cuMemAlloc(&d_norm, npad * (dc / 4) * sizeof(double)));
            void* na[] = {&d_data, &d_norm, &npad_u};
            CK(cuLaunchKernel(knorm, nb_tmp, 1, 1, 256, 1, 1, 0, 0, na, nullptr));
        }
        CK(cuMemAlloc(&d_n, sizeof(unsigned)));
        CK(cuMemcpyHtoD(d_n, &n, sizeof(unsigned)));
        CK(cuMemAlloc(&d_cnt, sizeof(unsigned long long)));
        CK(cuMemsetD8(d_cnt, 0, sizeof(unsigned long long)));
        CK(cuMemAlloc(&d_eps, sizeof(double)));
        const float eps32 = (float)eps;
        if (kind == "mq16") CK(cuMemcpyHtoD(d_eps, &eps32, sizeof(float)));
        else CK(cuMemcpyHtoD(d_eps, &eps, sizeof(double)));
        CK(cuEventRecord(e0, 0));
        if (kind == "cuda") {
            void* a[] = {&d_n, &d_data, &d_eps, &d_cnt};
            CK(cuLaunchKernel(kjoin, ceil_div(n, 256), 1, 1, 256, 1, 1, 0, 0, a, nullptr));
        } else if (kind == "mq16") {
            void* a[] = {&d_n, &d_alt, &d_eps, &d_cnt, &d_norm};
            CK(cuLaunchKernel(kjoin, ceil_div(2ull * n, 128), 1, 1, 128, 1, 1, 0, 0, a, nullptr));
        } else {
            void* a[] = {&d_n, &d_data, &d_eps, &d_cnt, &d_norm};
            CK(cuLaunchKernel(kjoin, ceil_div(4ull * n, 128), 1, 1, 128, 1, 1, 0, 0, a, nullptr));
        }
        CK(cuEventRecord(e1, 0));
        CK(cuCtxSynchronize());
        CK(cuMemcpyDtoH(&total, d_cnt, sizeof total));
        const auto t1 = std::chrono::steady_clock::now();
        float ms = 0.f;
        CK(cuEventElapsedTime(&ms, e0, e1));
        if (r > 0) {
            kms.push_back(ms);
            dms.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
        }
        for (CUdeviceptr p : {d_data, d_alt, d_norm, d_n, d_cnt, d_eps})
            if (p) CK(cuMemFree(p));
    }
    auto mean = [](const std::vector<double>& v) {
        double s = 0;
        for (double x : v) s += x;
        return v.empty() ? 0.0 : s / v.size();
    };
    auto best = [](const std::vector<double>& v) {
        return v.empty() ? 0.0 : *std::min_element(v.begin(), v.end());
    };
    printf("{\"kind\": \"%s\", \"cubin\": \"%s\", \"n\": %u, \"input_dim\": %u, \"compute_dim\": %u, "
           "\"eps\": %.17g, \"total\": %llu, \"kernel_ms_best\": %.6f, \"kernel_ms_mean\": %.6f, "
           "\"driver_ms_best\": %.6f, \"driver_ms_mean\": %.6f, \"reps\": %d}\n",
           kind.c_str(), cubin, n, din, dc, eps, total, best(kms), mean(kms), best(dms), mean(dms),
           reps);
    CK(cuModuleUnload(mod));
    CK(cuDevicePrimaryCtxRelease(dev));
    return 0;
}
