/*
 * ejoin_compat.h -- source-compatible replacement for the reference's
 * gpu_join.h (gpu_join.h:36-42 declares GPUJoinMainBruteForce).
 *
 * A program written against the reference (its main.cu:94 calls
 * GPUJoinMainBruteForce) includes this header instead of gpu_join.h, keeps
 * its params.h, and links libejoin.so instead of gpu_join.cu/kernel_join.cu.
 * The wrapper forwards the compile-time INPUT_DATA_DIM / COMPUTE_DIM of that
 * params.h to the run-time entry point.  The exact FP64 predicate needs FP64
 * input and eps, i.e. the reference's INPUT_DATA_PREC 64 / ACCUM_PREC 64
 * configuration; the FP32-eps overload below covers the shipped
 * ACCUM_PREC 32 configuration (eps widened exactly to double).
 */
#ifndef EJOIN_COMPAT_H
#define EJOIN_COMPAT_H

#include <stdint.h>
#include <stdio.h>

#include "ejoin.h"

#ifndef INPUT_DATA_DIM
#error "include the program's params.h (INPUT_DATA_DIM, COMPUTE_DIM) before ejoin_compat.h"
#endif

static inline void GPUJoinMainBruteForce(unsigned int searchMode, unsigned int device,
                                         double* dataset, unsigned int* nbQueryPoints,
                                         double* epsilon, uint64_t* totalNeighbors)
{
    int rc = ejoin_gpu_join_main_brute_force(searchMode, device, dataset, nbQueryPoints,
                                             epsilon, totalNeighbors, INPUT_DATA_DIM,
                                             COMPUTE_DIM);
    if (rc != EJOIN_OK) {
        char msg[512];
        ejoin_last_error(msg, sizeof msg);
        fprintf(stderr, "[GPU] ~ Error: %s\n", msg);
    }
}

#ifdef __cplusplus
static inline void GPUJoinMainBruteForce(unsigned int searchMode, unsigned int device,
                                         double* dataset, unsigned int* nbQueryPoints,
                                         float* epsilon, uint64_t* totalNeighbors)
{
    double eps = (double)*epsilon;
    GPUJoinMainBruteForce(searchMode, device, dataset, nbQueryPoints, &eps, totalNeighbors);
}
#endif

#endif /* EJOIN_COMPAT_H */
