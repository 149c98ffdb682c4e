/*
 * ejoin_testing.h -- test hooks of libejoin.so (not part of the join API).
 *
 * No reference counterpart: the learned projection is new.  These entry
 * points run single building blocks of the projection training on the GPU
 * so that the test-suite can compare them with a CPU restatement.
 */
#ifndef EJOIN_TESTING_H
#define EJOIN_TESTING_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One forward + hinge-loss + backward pass of the training kernel over M
 * pairs: V (M x d FP32 differences), tgt (M hinge targets; 0 = inactive),
 * P (k x d FP32).  Writes dL/dP (k x d) to G_out and the loss to *loss_out.
 * All pointers are host memory.  Returns 0 or a negative EJOIN_E* status. */
int ejoin_testing_projection_grad(const float* V, const float* tgt, uint64_t M, const float* P,
                                  uint32_t k, uint32_t d, float* G_out, float* loss_out);

/* Power-iteration renormalisation step on a host k x d matrix (in place);
 * *sigma_est_out receives the inflated estimate the kernel used. */
int ejoin_testing_renormalise(float* P, uint32_t k, uint32_t d, float* sigma_est_out);

/* Failure injection for the tests of the error paths.  The reference
 * printed CUDA errors and carried on (utils.cu:7-13) or exited
 * (gpu_join.cu:313-314, dataset.cu:16-20); here every failure returns a
 * status, and these hooks make the failures happen on purpose, on the host
 * side of the library, so that the tests can check the status, that every
 * buffer is released and that the next call succeeds.
 *   EJOIN_TESTING_FAIL_ALLOC    value = k: the k-th device allocation from
 *                               now fails (EJOIN_ENOMEM); 0 cancels
 *   EJOIN_TESTING_GRAM_TIMEOUT  value = ns: the next tensor-core screen runs
 *                               with that wait deadline and a producer that
 *                               never issues its first stage, so its bounded
 *                               waits expire (EJOIN_ETIMEOUT); 0 cancels
 * Process-wide; each injection is used once. */
#define EJOIN_TESTING_FAIL_ALLOC 1
#define EJOIN_TESTING_GRAM_TIMEOUT 2
int ejoin_testing_inject(int what, uint64_t value);

#ifdef __cplusplus
}
#endif

#endif /* EJOIN_TESTING_H */
