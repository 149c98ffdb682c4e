// cli_main.cpp -- command-line driver with the reference's interface.
//
// Same positional arguments as the reference's main (main.cu:17-26, ids in
// params.h:160-171):
//     ejoin_main <dataset> <epsilon> <searchMode> [device] [--dim D] [--binary] [--precision P]
// searchMode 1/2 = exact FP64 arbiter, 3/4 = exact tensor-core join, 5 = with
// learned pruning.  The reference fixed the dimension at compile time
// (INPUT_DATA_DIM, params.h:4); here it is --dim (default: the number of
// values on the first line of the file).  The result is appended to
// tensor_brute-force.txt in the reference's CSV format (main.cu:115-127:
// header written when the file is empty), with the dataset, epsilon,
// searchMode, join time, total, input dim, compute dim, block size, warps
// per block, compute and accumulation precision columns.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <fstream>
#include <iostream>
#include <string>

#include "ejoin.h"

static unsigned first_line_values(const char* path) {
    FILE* f = fopen(path, "r");
    if (!f) return 0;
    char buf[1 << 16];
    unsigned count = 0;
    if (fgets(buf, sizeof buf, f)) {
        char* p = buf;
        for (;;) {
            while (*p == ' ' || *p == '\t' || *p == ',') ++p;
            char* end = nullptr;
            strtod(p, &end);
            if (end == p) break;
            ++count;
            p = end;
        }
    }
    fclose(f);
    return count;
}

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr,
                "usage: %s <dataset> <epsilon> <searchMode> [device] [--dim D] [--binary] "
                "[--precision fp64_direct|fp64_dmma|fp16|bf16|bf16_split|auto]\n",
                argv[0]);
        return 1;
    }
    const char* filename = argv[1];
    const double epsilon = atof(argv[2]);
    const unsigned searchMode = (unsigned)atoi(argv[3]);
    unsigned device = 0;
    unsigned dim = 0;
    bool binary = false;
    int precision = -1;
    for (int i = 4; i < argc; ++i) {
        if (!strcmp(argv[i], "--dim") && i + 1 < argc) dim = (unsigned)atoi(argv[++i]);
        else if (!strcmp(argv[i], "--binary")) binary = true;
        else if (!strcmp(argv[i], "--precision") && i + 1 < argc) {
            const char* p = argv[++i];
            const char* names[] = {"fp64_direct", "fp64_dmma", "fp16", "bf16", "bf16_split", "fp8_e4m3", "auto"};
            for (int k = 0; k < 7; ++k)
                if (!strcmp(p, names[k])) precision = k;
        } else if (i == 4) device = (unsigned)atoi(argv[i]);
    }
    if (!dim) dim = binary ? 0 : first_line_values(filename);
    if (!dim) {
        fprintf(stderr, "[Main] ~ Error: give the dimension with --dim\n");
        return 1;
    }

    double* points = nullptr;
    uint64_t n = 0;
    const auto t0 = std::chrono::steady_clock::now();
    int rc = binary ? ejoin_import_binary(filename, dim, &points, &n)
                    : ejoin_import_dataset(filename, dim, &points, &n);
    const auto t1 = std::chrono::steady_clock::now();
    if (rc != EJOIN_OK) {
        char msg[512];
        ejoin_last_error(msg, sizeof msg);
        fprintf(stderr, "%s\n", msg);
        return 1;
    }
    std::cout << "[Main | Time] ~ Time to read the dataset: "
              << std::chrono::duration<double>(t1 - t0).count() << '\n';

    ejoin_options opt;
    ejoin_default_options(&opt);
    opt.device = (int)device;
    switch (searchMode) {
        case 1: case 2: opt.precision = EJOIN_FP64_DIRECT; break;
        case 3: case 4: opt.precision = EJOIN_AUTO; break;
        case 5: opt.precision = EJOIN_AUTO; opt.proj_k = 8; break;
        default:
            std::cerr << "[Main] ~ Error: Unknown search mode\n";
            ejoin_free(points);
            return 1;
    }
    if (precision >= 0) opt.precision = precision;
    uint64_t total = 0;
    ejoin_stats st;
    const auto t2 = std::chrono::steady_clock::now();
    rc = ejoin_self_join(points, n, dim, epsilon, &opt, nullptr, &total, &st);
    const auto t3 = std::chrono::steady_clock::now();
    ejoin_free(points);
    if (rc != EJOIN_OK) {
        char msg[512];
        ejoin_last_error(msg, sizeof msg);
        fprintf(stderr, "[GPU] ~ Error: %s\n", msg);
        return 1;
    }
    const double timeJoin = std::chrono::duration<double>(t3 - t2).count();
    std::cout << "[Main | Result] ~ Time to join: " << timeJoin << '\n';
    std::cout << "[Main | Result] ~ Total result set size: " << total << '\n';

    // CSV line of the reference (main.cu:115-127).  The reference wrote its
    // compile-time COMPUTE_DIM, BLOCKSIZE, WARP_PER_BLOCK and precisions; here
    // the columns describe the main kernel of the mode actually run (the
    // library reports it in st.precision):
    //   FP64 direct   d coordinates, 256-thread blocks (8 warps)
    //   FP64 DMMA     d padded to 32, 128-thread CTAs (4 warps)
    //   16-bit Gram   d padded to 64, 608-thread CTAs (19 warps)
    //   FP8 Gram      d padded to 128, 608-thread CTAs (19 warps)
    const char* precs[] = {"64", "64", "16", "16", "16", "8", "16"};
    const int pm = st.precision >= 0 && st.precision <= 6 ? st.precision : 6;
    unsigned computeDim = (dim + 63) / 64 * 64, blockSize = 608, warps = 19;
    if (pm == EJOIN_FP64_DIRECT) {
        computeDim = dim;
        blockSize = 256;
        warps = 8;
    } else if (pm == EJOIN_FP64_DMMA) {
        computeDim = (dim + 31) / 32 * 32;
        blockSize = 128;
        warps = 4;
    } else if (pm == EJOIN_FP8_E4M3) {
        computeDim = (dim + 127) / 128 * 128;
    }
    std::ofstream out;
    std::ifstream in("tensor_brute-force.txt");
    const bool empty = !in.good() || in.peek() == std::ifstream::traits_type::eof();
    out.open("tensor_brute-force.txt", std::ios::out | std::ios::app);
    if (empty)
        out << "Dataset, epsilon, searchMode, executionTime, totalNeighbors, inputDim, computeDim, "
               "blockSize, warpPerBlock, computePrec, accumPrec\n";
    out << filename << ", " << epsilon << ", " << searchMode << ", " << timeJoin << ", " << total
        << ", " << dim << ", " << computeDim << ", " << blockSize << ", " << warps << ", "
        << precs[pm] << ", " << (pm <= 1 ? 64 : 32) << std::endl;
    return 0;
}
