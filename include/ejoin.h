/*
 * ejoin.h -- C ABI of libejoin.so, the GB300 (sm_103a) exact epsilon self-join.
 *
 * Given n points of dimension d (FP64, row-major) and a radius eps, the join
 * counts for every point i the points j with sqrt(d2(i, j)) <= eps, where
 * d2 is formed exactly as the reference's FP64 CUDA-core kernel forms it
 * (kernel_join.cu:184-199 of the reference: per coordinate t = a - b, then
 * acc = fma(t, t, acc) in index order).  Self pairs are included, so the
 * total is the number of ordered pairs, the reference's totalNeighbors.
 *
 * Every precision mode returns counts bit-identical to that FP64 predicate:
 * the fast modes screen pairs with tensor-core Gram products and a rigorous
 * per-pair error bound, and recompute only the pairs inside the boundary band
 * in FP64 with the reference arithmetic.
 *
 * All entry points return 0 on success or a negative EJOIN_E* status; none
 * exits or aborts.  ejoin_last_error() describes the last failure of the
 * calling thread.  The library allocates and frees its own device scratch;
 * the caller owns inputs and outputs.
 */
#ifndef EJOIN_H
#define EJOIN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EJOIN_VERSION_MAJOR 1
#define EJOIN_VERSION_MINOR 0

/* status codes */
#define EJOIN_OK 0
#define EJOIN_EINVAL (-1)        /* bad argument */
#define EJOIN_ECUDA (-2)         /* CUDA runtime / driver error */
#define EJOIN_ENOMEM (-3)        /* device or host allocation failed */
#define EJOIN_ENODEV (-4)        /* no usable sm_103 device */
#define EJOIN_EUNSUPPORTED (-5)  /* mode / size combination not supported */
#define EJOIN_ETIMEOUT (-6)      /* a bounded device-side wait expired */
#define EJOIN_EIO (-7)           /* file could not be opened / read */
#define EJOIN_EINTERNAL (-8)     /* internal consistency check failed */

/* Precision modes (the reference chose precision at compile time through
 * INPUT_DATA_PREC / COMPUTE_PREC / ACCUM_PREC, params.h:10-12 and
 * params.h:175-203; here it is a runtime option). */
typedef enum ejoin_precision {
    EJOIN_FP64_DIRECT = 0, /* CUDA-core direct differences: the exact arbiter
                              (reference searchMode 1, kernel_join.cu:168-200) */
    EJOIN_FP64_DMMA = 1,   /* FP64 DMMA Gram tiles + FP64 band recheck
                              (reference kernel_join.cu:530-677 re-designed) */
    EJOIN_FP16 = 2,        /* tcgen05 kind::f16, FP16 operands, FP32 accumulate */
    EJOIN_BF16 = 3,        /* tcgen05 kind::f16, BF16 operands, FP32 accumulate */
    EJOIN_BF16_SPLIT = 4,  /* BF16 hi+lo split products (hi*hi + hi*lo + lo*hi) */
    EJOIN_FP8_E4M3 = 5,    /* tcgen05 kind::f8f6f4, E4M3 with per-row scales */
    EJOIN_AUTO = 6         /* library picks (FP16 for d <= 128, else BF16) */
} ejoin_precision;

/* Point ordering used by the learned pruning (proj_k > 0). */
typedef enum ejoin_order {
    EJOIN_ORDER_MORTON = 0, /* Morton (Z-order) key over the projected coords */
    EJOIN_ORDER_LEAD = 1    /* sort by the leading projected coordinate only */
} ejoin_order;

typedef struct ejoin_options {
    uint32_t struct_size;     /* sizeof(ejoin_options); set by ejoin_default_options */
    int32_t device;           /* CUDA device ordinal (default 0) */
    int32_t precision;        /* ejoin_precision (default EJOIN_AUTO) */
    uint32_t proj_k;          /* learned projection rows; 0 = plain join, no pruning */
    uint64_t ld;              /* row stride of `points` in elements (0 = d) */
    const float* projection;  /* optional host k x d projection to reuse (skips
                                 training); its spectral norm is re-certified */
    uint64_t train_pairs;     /* pairs sampled for training (default 1<<19) */
    uint32_t train_steps;     /* optimiser steps (default 50: longer training lowers the
                                 hinge loss but not the number of pruned tile pairs) */
    uint32_t order;           /* ejoin_order (default MORTON) */
    uint64_t seed;            /* seed for sampling / initialisation */
    void* stream;             /* cudaStream_t to run on (NULL = library stream) */
    uint64_t band_capacity;   /* band-queue entries (0 = automatic, grows on overflow) */
    double acc_bound_scale;   /* multiplier on the tensor-core accumulation error
                                 bound (default 1.0; values < 1 are rejected) */
    uint32_t flags;           /* EJOIN_FLAG_* */
    uint32_t reserved[7];
} ejoin_options;

#define EJOIN_FLAG_NO_RECHECK_STATS 0x1u /* reserved */
/* Keep the device scratch cached in the library's memory pool after the call,
 * so that repeated joins skip the cost of mapping fresh device memory.
 * Without it every call returns its scratch to the device before it returns
 * (the library never touches the device's default pool).  The cached memory
 * is released by ejoin_release_scratch or at exit. */
#define EJOIN_FLAG_KEEP_SCRATCH 0x2u

typedef struct ejoin_stats {
    uint64_t n;
    uint32_t d;
    int32_t precision;          /* the mode actually run */
    uint64_t band_pairs;        /* directed pairs sent to the FP64 recheck */
    uint64_t band_hits;         /* band pairs that turned out to be neighbours */
    uint64_t tile_pairs_total;  /* upper-triangle tile pairs of the plain join */
    uint64_t tile_pairs_run;    /* tile pairs that reached the Gram kernel */
    uint64_t band_overflows;    /* band-queue overflows (each forced a re-run) */
    double band_fraction;       /* band_pairs / ordered pairs computed */
    double sigma_cert;          /* certified upper bound of ||P||_2 (learned mode) */
    double ms_total;            /* device time of the whole join */
    double ms_prep;             /* centring, norms, packing */
    double ms_train;            /* projection training + certification */
    double ms_order;            /* projection, sort, tile boxes, survivor list */
    double ms_gram;             /* the Gram / direct kernel */
    double ms_recheck;          /* FP64 band recheck */
    double gram_flops;          /* MMA (or FP64) flops executed by the Gram kernel */
    uint64_t kernel_launches;   /* CUDA kernels this call launched */
    /* reserved[0]: band pairs the FP32 pre-check left to the exact FP64 chain;
       reserved[1]: 128 x 256 blocks the tensor-core Gram kernel computed
       (each covers up to two of the tile_pairs_run 128 x 128 tile pairs);
       reserved[2]: peak device scratch the call reserved (bytes);
       reserved[3]: band records the tensor-core Gram kernel wrote (one per row
       and 32-column chunk with band pairs, 16 bytes each);
       ejoin_train_projection: reserved[0] / [1] = first / last hinge loss. */
    double reserved[5];
} ejoin_stats;

/* Fill *opt with defaults. */
int ejoin_default_options(ejoin_options* opt);

/* The exact self-join.
 *   points     row-major n x d FP64 (row stride opt->ld), host or device memory
 *   counts_out n int32 per-point counts (self included), host or device, may be NULL
 *   total_out  sum of the counts (ordered pairs), may be NULL
 *   stats_out  may be NULL
 * Replaces the reference's GPUJoinMainBruteForce (gpu_join.cu:210-322,
 * declared gpu_join.h:36-42), which returned only the total. */
int ejoin_self_join(const double* points, uint64_t n, uint32_t d, double eps,
                    const ejoin_options* opt, int32_t* counts_out, uint64_t* total_out,
                    ejoin_stats* stats_out);

/* Neighbour lists of the exact self-join (CSR): the points j with
 * sqrt(d2(i, j)) <= eps for every point i in input order, ascending, i itself
 * included -- list i has the length ejoin_self_join reports as count i.
 *   offsets    n + 1 entries: list i is neighbors[offsets[i] .. offsets[i+1])
 *   neighbors  capacity entries, may be NULL (then only offsets and the total
 *              are computed); if capacity is below the total, offsets and
 *              *total_out are filled, neighbors is not written and
 *              EJOIN_ENOMEM is returned (call again with a larger buffer)
 * Host or device pointers.  The total must stay below 2^31.  No reference
 * counterpart: the reference returns only the total (gpu_join.cu:210-322);
 * its result-set kernels (kernel_join.cu:139-162) are dead code. */
int ejoin_neighbor_lists(const double* points, uint64_t n, uint32_t d, double eps,
                         const ejoin_options* opt, uint64_t* offsets, uint32_t* neighbors,
                         uint64_t capacity, uint64_t* total_out, ejoin_stats* stats_out);

/* Join of two point sets: for every query row q, the number of points j with
 * sqrt(d2(q, x_j)) <= eps (d2 formed as the reference's FP64 kernel forms it,
 * kernel_join.cu:168-200).  queries nq x d and points n x d, row-major with
 * the same row stride opt->ld, host or device; counts_out nq int32 (host or
 * device, may be NULL); total_out their sum.  Same precision modes as
 * ejoin_self_join, counts exact in every mode; opt->proj_k must be 0.  No
 * reference counterpart (the reference joins a set with itself only). */
int ejoin_join_counts(const double* queries, uint64_t nq, const double* points, uint64_t n,
                      uint32_t d, double eps, const ejoin_options* opt, int32_t* counts_out,
                      uint64_t* total_out, ejoin_stats* stats_out);

/* Counts for the query rows `rows[0..nq)` against all n points (same exact
 * predicate), computed with the FP64 direct kernel.  Used to check sampled
 * rows of large joins.  No reference counterpart (the reference has no
 * per-point output). */
int ejoin_query_counts(const double* points, uint64_t n, uint32_t d, double eps,
                       const uint64_t* rows, uint64_t nq, const ejoin_options* opt,
                       int32_t* counts_out);

/* Train the contractive projection P (k x d, row-major FP32, written to the
 * host buffer P_out) on pairs sampled from the join, and return the certified
 * upper bound of its spectral norm (<= 1 after renormalisation).  No
 * reference counterpart (the learned pruning is new). */
int ejoin_train_projection(const double* points, uint64_t n, uint32_t d, double eps,
                           const ejoin_options* opt, float* P_out, double* sigma_cert_out,
                           ejoin_stats* stats_out);

/* Certified upper bound of the spectral norm of a host k x d FP32 matrix
 * (host arithmetic, rigorous). */
int ejoin_certify_spectral_norm(const float* P, uint32_t k, uint32_t d, double* bound_out);

/* Return the device scratch cached by calls made with EJOIN_FLAG_KEEP_SCRATCH
 * on `device` to the device.  No reference counterpart (the reference never
 * freed its device memory, gpu_join.cu:210-322). */
int ejoin_release_scratch(int device);

/* Largest double T with sqrt(T) <= eps: the join counts pairs with d2 <= T. */
double ejoin_threshold(double eps);

/* Text loader with the reference's semantics (dataset.cu:10-39): numbers
 * separated by commas and/or whitespace, a row closes every `dim` values, a
 * trailing partial row is dropped.  *points_out is allocated by the library
 * -- page-locked host memory where a CUDA device is present, so that a join
 * from it copies in chunks overlapped with its first passes -- and freed with
 * ejoin_free.  Returns EJOIN_EIO if the file cannot be opened (the reference
 * printed and exited, dataset.cu:16-20). */
int ejoin_import_dataset(const char* filename, uint32_t dim, double** points_out,
                         uint64_t* n_out);

/* Binary loader: raw little-endian float64, row-major, `dim` columns, read
 * in 64 MiB pieces straight into the result (allocated as for
 * ejoin_import_dataset).  The fast path for the 1-8 GB inputs whose text form
 * the reference's fscanf loop (dataset.cu:25-36) takes minutes to parse. */
int ejoin_import_binary(const char* filename, uint32_t dim, double** points_out,
                        uint64_t* n_out);

/* Free a buffer returned by the loaders. */
void ejoin_free(void* p);

/* Save a learned projection (k x d FP32, row-major, 1 <= k <= 16) with its
 * certified spectral-norm bound to a small binary file (magic, version, k, d,
 * bound, the values, a checksum), for reuse by later joins through
 * ejoin_options.projection.  No reference counterpart (the projection is
 * new; the reference keeps no state between runs). */
int ejoin_save_projection(const char* filename, const float* P, uint32_t k, uint32_t d,
                          double sigma_cert);

/* Load a projection saved by ejoin_save_projection.  With P_out NULL only the
 * shape (and bound) is returned; else P_out must hold capacity >= k * d
 * floats.  A file that is not a projection file, has another version, the
 * wrong size or a bad checksum returns EJOIN_EIO. */
int ejoin_load_projection(const char* filename, float* P_out, uint64_t capacity, uint32_t* k_out,
                          uint32_t* d_out, double* sigma_cert_out);

/* Copy the calling thread's last error message into buf (NUL-terminated);
 * returns the status of that error (0 if none). */
int ejoin_last_error(char* buf, size_t len);

/* Library version as major * 100 + minor. */
int ejoin_version(void);

/* Drop-in for the reference driver GPUJoinMainBruteForce (gpu_join.cu:210-216):
 * same arguments, plus the reference's compile-time INPUT_DATA_DIM and
 * COMPUTE_DIM (params.h:4-5) passed at run time.  `dataset` is the padded
 * host array (row stride compute_dim, input_dim columns used) that main.cu:38-57
 * builds; *nbQueryPoints is N (the 15 zero rows of padding are ignored).
 * searchMode: 1 (SM_GPU) and 2 (SM_CUDA_ALT) run EJOIN_FP64_DIRECT, 3
 * (SM_TENSOR) and 4 (SM_TENSOR_MQ) run the exact tensor-core join
 * (EJOIN_AUTO), 5 runs it with learned pruning (k = 8).  Unlike the
 * reference, the result is exact, the counter is zeroed, device memory is
 * freed and an unknown mode returns EJOIN_EINVAL instead of exiting.
 * ejoin_compat.h wraps this as GPUJoinMainBruteForce with the reference's
 * exact signature. */
int ejoin_gpu_join_main_brute_force(unsigned int searchMode, unsigned int device,
                                    double* dataset, unsigned int* nbQueryPoints,
                                    double* epsilon, uint64_t* totalNeighbors,
                                    unsigned int input_dim, unsigned int compute_dim);

/* Exact self-join that allocates no device memory, for callers that cannot
 * call cudaMalloc while they run the join (an engine that owns all device
 * memory through its own pool, a serving path that forbids allocation and
 * its implicit synchronisation, a process under a hard memory cap).  No
 * counterpart in the reference.  It runs the FP64 DMMA screen and the FP64
 * band recheck (counts identical to ejoin_self_join) with all scratch in one
 * static 32 MiB device array that every GPU loading the library holds until
 * exit.  Limits: n <= 16384, d <= 128 (else EJOIN_EINVAL); a boundary band
 * larger than the array's queue returns EJOIN_ENOMEM.  `points` (n x d,
 * contiguous) and `counts` (n int32) must be device memory of `device` (or
 * managed memory), else EJOIN_EINVAL before any launch; *total_out is host
 * memory (may be NULL); `stream` may be NULL.  Every call waits for its own
 * work on `stream` before returning (the status and total are read back to
 * the host).  On a non-zero return the counts are zero.  The first call on a
 * device resolves the array's address and should come before any stream
 * capture on that device.  All calls share the array: calls that overlap on
 * the GPU race. */
int ejoin_self_join_noalloc(const double* points, uint64_t n, uint32_t d, double eps,
                            int device, void* stream, int32_t* counts, uint64_t* total_out);

#ifdef __cplusplus
}
#endif

#endif /* EJOIN_H */
