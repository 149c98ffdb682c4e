/*
 * oracle.c -- CPU restatement of the reference's brute-force epsilon self-join.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests,
 * __graft_entry__.smoke() and the cpu_baseline / reference legs of bench.py
 * load it.  The product (libejoin.so) never links, loads or calls it.
 *
 * What it restates (reference paths are relative to the reference project):
 *
 *  - kernel_join.cu:168-200 `distanceCalculationBruteForceCuda` (searchMode 1,
 *    the FP64 CUDA-core kernel): for a query p and candidate c,
 *        acc = 0; for j in 0..d-1: acc += (p_j - c_j) * (p_j - c_j)
 *    in double, index order (kernel_join.cu:185-189); then a pair is a
 *    neighbour iff sqrt(acc) <= eps (kernel_join.cu:194).  Every ordered pair
 *    (i, j) is tested, the self pair included (the loop at :184 runs over all
 *    points).  How the products are rounded is the compiler's choice; the
 *    reference's kernel compiled by nvcc for sm_103a computes, with
 *    t_j = fl(p_j - c_j),
 *        acc = fma(t_0, t_0, fl(t_1 * t_1));  acc = fma(t_j, t_j, acc), j >= 2
 *    (`0 + t_0 * t_0` folds into the bare product, which is then fused into
 *    the second step).  That form was pinned by running the reference's own
 *    compiled kernel (built from its sources by oracle/build_ref.sh) on
 *    pairs within ulps of the radius that the plain fma chain, this form and
 *    the uncontracted sum count differently (tests/golden/contraction*.json),
 *    at d = 18, 64 and 128.  This file writes every fma explicitly and is
 *    compiled with -ffp-contract=off so no other contraction can happen.
 *
 *  - The predicate sqrt(acc) <= eps is evaluated as acc <= T where T is the
 *    largest double whose correctly rounded square root is <= eps
 *    (oracle_threshold).  IEEE sqrt is correctly rounded and monotone, so the
 *    two tests agree for every acc, NaN included (NaN <= T is false, as
 *    sqrt(NaN) <= eps is false).
 *
 *  - dataset.cu:10-39 `importDataset`: the fscanf("%lf, ") / fscanf("%lf ")
 *    loop that closes a row every `dim` values and drops a trailing partial
 *    row (oracle_import_dataset).
 *
 * Per-point counts are an addition of the new interface; their sum is the
 * reference's total (the single 64-bit counter of gpu_join.cu:261-263,320).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#if defined(__FP_FAST_FMA) || defined(__aarch64__)
#define ORACLE_HW_FMA 1
#else
#define ORACLE_HW_FMA 0
#endif

/* Largest double T with sqrt(T) <= eps (IEEE correctly rounded sqrt).
 * eps NaN -> NaN (no pair qualifies); eps < 0 -> -inf (no pair qualifies);
 * eps = +inf -> +inf. */
double oracle_threshold(double eps)
{
    if (isnan(eps)) return NAN;
    if (eps < 0.0) return -INFINITY;           /* -0.0 is not < 0 */
    if (isinf(eps)) return INFINITY;
    double t = eps * eps;
    if (isinf(t)) t = 1.7976931348623157e308;
    while (t > 0.0 && sqrt(t) > eps) t = nextafter(t, 0.0);
    for (;;) {
        double up = nextafter(t, INFINITY);
        if (isinf(up) || !(sqrt(up) <= eps)) break;
        t = up;
    }
    return t;
}

/* Squared distance exactly as the reference's FP64 kernel computes it once
 * compiled (see the header): fma(t0, t0, fl(t1 * t1)), then fma(t, t, acc). */
static inline double pair_d2(const double* a, const double* b, uint32_t d)
{
    double t0 = a[0] - b[0];
    double t1 = d > 1 ? a[1] - b[1] : 0.0;
    double acc = fma(t0, t0, t1 * t1);
    for (uint32_t k = 2; k < d; ++k) {
        double t = a[k] - b[k];
        acc = fma(t, t, acc);
    }
    return acc;
}

/* Four independent chains at once: identical arithmetic per chain, only the
 * interleaving differs (for instruction-level parallelism on the CPU). */
static inline void pair_d2_x4(const double* a, const double* b0, const double* b1,
                              const double* b2, const double* b3, uint32_t d,
                              double out[4])
{
    double s0, s1, s2, s3;
    {
        double a0 = a[0], a1 = d > 1 ? a[1] : 0.0;
        double u0 = a0 - b0[0], u1 = a0 - b1[0], u2 = a0 - b2[0], u3 = a0 - b3[0];
        double v0 = d > 1 ? a1 - b0[1] : 0.0, v1 = d > 1 ? a1 - b1[1] : 0.0;
        double v2 = d > 1 ? a1 - b2[1] : 0.0, v3 = d > 1 ? a1 - b3[1] : 0.0;
        s0 = fma(u0, u0, v0 * v0);
        s1 = fma(u1, u1, v1 * v1);
        s2 = fma(u2, u2, v2 * v2);
        s3 = fma(u3, u3, v3 * v3);
    }
    for (uint32_t k = 2; k < d; ++k) {
        double ak = a[k];
        double t0 = ak - b0[k], t1 = ak - b1[k], t2 = ak - b2[k], t3 = ak - b3[k];
        s0 = fma(t0, t0, s0);
        s1 = fma(t1, t1, s1);
        s2 = fma(t2, t2, s2);
        s3 = fma(t3, t3, s3);
    }
    out[0] = s0; out[1] = s1; out[2] = s2; out[3] = s3;
}

double oracle_pair_d2(const double* a, const double* b, uint32_t d)
{
    return pair_d2(a, b, d);
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int oracle_hw_fma(void) { return ORACLE_HW_FMA; }

/* Count, for each query row q in `rows` (or rows 0..nq-1 when rows == NULL),
 * the points j in 0..n-1 with d2(x_q, x_j) <= T.  x is row-major with row
 * stride ld (>= d) elements. */
int oracle_query_counts(const double* x, uint64_t n, uint32_t d, uint64_t ld,
                        double eps, const uint64_t* rows, uint64_t nq,
                        int32_t* counts, int nthreads)
{
    if (!x && n) return -1;
    if (ld < d) return -2;
    const double T = oracle_threshold(eps);
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int64_t qi = 0; qi < (int64_t)nq; ++qi) {
        const uint64_t q = rows ? rows[qi] : (uint64_t)qi;
        const double* a = x + q * ld;
        int64_t c = 0;
        uint64_t j = 0;
        double d2[4];
        for (; j + 4 <= n; j += 4) {
            pair_d2_x4(a, x + j * ld, x + (j + 1) * ld, x + (j + 2) * ld, x + (j + 3) * ld, d, d2);
            c += (d2[0] <= T) + (d2[1] <= T) + (d2[2] <= T) + (d2[3] <= T);
        }
        for (; j < n; ++j) c += (pair_d2(a, x + j * ld, d) <= T);
        counts[qi] = (int32_t)c;
    }
    (void)nthreads;
    return 0;
}

/* Join of two point sets: for every query row q (nq x d, stride ld), the
 * points x_j (n x d, stride ld) with d2(q, x_j) <= T, the same chain as the
 * self-join ((q - x)^2 and (x - q)^2 are bitwise equal). */
int oracle_cross_counts(const double* q, uint64_t nq, const double* x, uint64_t n, uint32_t d,
                        uint64_t ld, double eps, int32_t* counts, int nthreads)
{
    if ((!q && nq) || (!x && n)) return -1;
    if (ld < d) return -2;
    const double T = oracle_threshold(eps);
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int64_t qi = 0; qi < (int64_t)nq; ++qi) {
        const double* a = q + (uint64_t)qi * ld;
        int64_t c = 0;
        uint64_t j = 0;
        double d2[4];
        for (; j + 4 <= n; j += 4) {
            pair_d2_x4(a, x + j * ld, x + (j + 1) * ld, x + (j + 2) * ld, x + (j + 3) * ld, d, d2);
            c += (d2[0] <= T) + (d2[1] <= T) + (d2[2] <= T) + (d2[3] <= T);
        }
        for (; j < n; ++j) c += (pair_d2(a, x + j * ld, d) <= T);
        counts[qi] = (int32_t)c;
    }
    (void)nthreads;
    return 0;
}

/* Full self-join: per-point counts (self included) and their uint64 sum. */
int oracle_self_join(const double* x, uint64_t n, uint32_t d, uint64_t ld, double eps,
                     int32_t* counts, uint64_t* total, int nthreads)
{
    int rc = oracle_query_counts(x, n, d, ld, eps, NULL, n, counts, nthreads);
    if (rc) return rc;
    uint64_t s = 0;
    for (uint64_t i = 0; i < n; ++i) s += (uint64_t)counts[i];
    if (total) *total = s;
    return 0;
}

/* Neighbour lists of the self-join (CSR): with offsets[] from the per-point
 * counts (offsets[i+1] - offsets[i] = count of row i), row i's entries are
 * the j in 0..n-1, ascending, with d2(x_i, x_j) <= T -- the predicate of
 * kernel_join.cu:194 restated as d2 <= T, the same chain as the counts. */
int oracle_neighbor_lists(const double* x, uint64_t n, uint32_t d, uint64_t ld, double eps,
                          const uint64_t* offsets, uint32_t* nb, int nthreads)
{
    if (!x && n) return -1;
    if (ld < d) return -2;
    const double T = oracle_threshold(eps);
    int overflow = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(|:overflow)
#endif
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const double* a = x + (uint64_t)i * ld;
        uint64_t o = offsets[i];
        for (uint64_t j = 0; j < n; ++j)
            if (pair_d2(a, x + j * ld, d) <= T) {
                if (o < offsets[i + 1]) nb[o] = (uint32_t)j;
                else overflow = 1;
                ++o;
            }
    }
    (void)nthreads;
    return overflow ? -3 : 0;
}

/* Restatement of dataset.cu:10-39.  Reads values with the same pair of
 * fscanf formats, closes a row every `dim` values and drops a trailing
 * partial row.  On success *out is a malloc'd row-major n x dim array
 * (free with oracle_free).  Returns -1 if the file cannot be opened
 * (the reference prints and exits, dataset.cu:16-20). */
int oracle_import_dataset(const char* filename, uint32_t dim, double** out, uint64_t* n_out)
{
    *out = NULL;
    *n_out = 0;
    if (dim == 0) return -2;
    FILE* f = fopen(filename, "r");
    if (!f) return -1;
    size_t cap = 1024, len = 0;
    double* buf = (double*)malloc(cap * sizeof(double));
    double v = 0;
    while (fscanf(f, "%lf, ", &v) == 1 || fscanf(f, "%lf ", &v) == 1) {
        if (len == cap) {
            cap *= 2;
            buf = (double*)realloc(buf, cap * sizeof(double));
        }
        buf[len++] = v;
    }
    fclose(f);
    uint64_t rows = len / dim;
    *out = buf;
    *n_out = rows;
    return 0;
}

void oracle_free(void* p) { free(p); }
