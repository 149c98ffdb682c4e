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

#ifdef __cplusplus
}
#endif

#endif /* EJOIN_TESTING_H */
