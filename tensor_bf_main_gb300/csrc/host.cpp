// host.cpp -- host-only parts of libejoin.so: the dataset loaders and the
// rigorous spectral-norm certificate of the learned projection.
#include <errno.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "ejoin.h"

namespace ejoin {
int set_error(int status, const char* fmt, ...);
void clear_error();
int cert_spectral_norm(const float* P, uint32_t k, uint32_t d, double* bound_out);
// api.cu: host buffers of the loaders, page-locked where a CUDA device is
// present (so that a join from them takes the chunked, overlapped copy)
void* host_alloc(size_t bytes);
}  // namespace ejoin

using ejoin::set_error;

namespace {

bool read_file(const char* filename, std::vector<char>& buf) {
    FILE* f = fopen(filename, "rb");
    if (!f) return false;
    buf.clear();
    char tmp[1 << 16];
    size_t r;
    while ((r = fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + r);
    fclose(f);
    buf.push_back('\0');
    return true;
}

inline bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// |A| * |B| style products for the interval squaring below
void matmul(const std::vector<double>& A, const std::vector<double>& B, std::vector<double>& C,
            int k) {
    C.assign((size_t)k * k, 0.0);
    for (int i = 0; i < k; ++i)
        for (int l = 0; l < k; ++l) {
            const double a = A[(size_t)i * k + l];
            for (int j = 0; j < k; ++j) C[(size_t)i * k + j] += a * B[(size_t)l * k + j];
        }
}

}  // namespace

extern "C" {

// Reference semantics (dataset.cu:10-39): the loop
//   while (fscanf(f, "%lf, ", &v) == 1 || fscanf(f, "%lf ", &v) == 1)
// reads a number after optional whitespace, then consumes a comma only if it
// immediately follows the number, then whitespace; it stops at the first
// token that is not a number.  Numbers are converted by strtod, the
// conversion fscanf's %lf uses.  A row closes every `dim` values; a trailing
// partial row is dropped.
int ejoin_import_dataset(const char* filename, uint32_t dim, double** points_out,
                         uint64_t* n_out) {
    ejoin::clear_error();
    if (!filename || !points_out || !n_out || dim == 0)
        return set_error(EJOIN_EINVAL, "bad arguments");
    *points_out = nullptr;
    *n_out = 0;
    std::vector<char> buf;
    if (!read_file(filename, buf))
        return set_error(EJOIN_EIO, "[Dataset] ~ Could not open the input file %s", filename);
    std::vector<double> vals;
    vals.reserve(buf.size() / 8);
    const char* p = buf.data();
    for (;;) {
        while (is_space(*p)) ++p;
        if (!*p) break;
        char* end = nullptr;
        errno = 0;
        const double v = strtod(p, &end);
        if (end == p) break;
        vals.push_back(v);
        p = end;
        if (*p == ',') {
            ++p;
            while (is_space(*p)) ++p;
        }
    }
    const uint64_t rows = vals.size() / dim;
    double* out = (double*)ejoin::host_alloc((rows ? rows : 1) * dim * sizeof(double));
    if (!out) return set_error(EJOIN_ENOMEM, "host allocation failed");
    if (rows) memcpy(out, vals.data(), rows * dim * sizeof(double));
    *points_out = out;
    *n_out = rows;
    return EJOIN_OK;
}

int ejoin_import_binary(const char* filename, uint32_t dim, double** points_out, uint64_t* n_out) {
    ejoin::clear_error();
    if (!filename || !points_out || !n_out || dim == 0)
        return set_error(EJOIN_EINVAL, "bad arguments");
    *points_out = nullptr;
    *n_out = 0;
    FILE* f = fopen(filename, "rb");
    if (!f) return set_error(EJOIN_EIO, "could not open %s", filename);
    fseek(f, 0, SEEK_END);
    const long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    const uint64_t rows = sz > 0 ? (uint64_t)sz / (8ull * dim) : 0;
    double* out = (double*)ejoin::host_alloc((rows ? rows : 1) * dim * sizeof(double));
    if (!out) {
        fclose(f);
        return set_error(EJOIN_ENOMEM, "host allocation failed");
    }
    // straight into the (page-locked) result, 64 MiB at a time
    const uint64_t total = rows * dim;
    uint64_t got = 0;
    while (got < total) {
        const size_t want = (size_t)std::min<uint64_t>(total - got, 8ull << 20);
        const size_t r = fread(out + got, sizeof(double), want, f);
        got += r;
        if (r != want) break;
    }
    fclose(f);
    if (got != total) {
        ejoin_free(out);
        return set_error(EJOIN_EIO, "short read on %s", filename);
    }
    *points_out = out;
    *n_out = rows;
    return EJOIN_OK;
}

// Certified upper bound of ||P||_2 for a k x d FP32 matrix.
//
// lambda_max(M)^(2^m) = lambda_max(M^(2^m)) <= ||M^(2^m)||_F for the PSD
// M = P P^T.  M is formed in FP64 (products of FP32 values are exact in
// FP64; the sums carry a radius gamma_d |P||P|^T) and squared m times in
// midpoint-radius arithmetic: with |T_s - A_s| <= R_s entrywise,
//   R_{s+1} = |A_s| R_s + R_s |A_s| + R_s R_s + gamma_k |A_s||A_s|
// encloses T_{s+1} - fl(A_s A_s).  Every step is rescaled by an exact power
// of two.  The bound (||A_m||_F + ||R_m||_F)^(1/2^m) overestimates sigma_max
// by at most a factor k^(1/2^(m+1)) (about 0.14% for k = 16, m = 10); all
// radius computations carry an extra relative margin for their own rounding.
int ejoin_certify_spectral_norm(const float* P, uint32_t k, uint32_t d, double* bound_out) {
    ejoin::clear_error();
    return ejoin::cert_spectral_norm(P, k, d, bound_out);
}

}  // extern "C"

namespace ejoin {

int cert_spectral_norm(const float* P, uint32_t k, uint32_t d, double* bound_out) {
    if (!P || !bound_out || k == 0 || d == 0 || k > 256)
        return set_error(EJOIN_EINVAL, "bad arguments");
    const double u = 1.1102230246251565e-16;
    const double gd = (d + 2) * u / (1 - (d + 2) * u);
    const double gk = (k + 2) * u / (1 - (k + 2) * u);
    const double marg = 1.0 + 8.0 * (k + d) * u;
    std::vector<double> A((size_t)k * k), R((size_t)k * k);
    for (uint32_t i = 0; i < k; ++i)
        for (uint32_t j = 0; j < k; ++j) {
            double s = 0.0, sa = 0.0;
            for (uint32_t c = 0; c < d; ++c) {
                const double pr = (double)P[(size_t)i * d + c] * (double)P[(size_t)j * d + c];
                if (!isfinite(pr)) return set_error(EJOIN_EINVAL, "projection has non-finite entries");
                s += pr;
                sa += fabs(pr);
            }
            A[(size_t)i * k + j] = s;
            R[(size_t)i * k + j] = gd * sa * marg;
        }
    double log2scale = 0.0;  // M^(2^s) = 2^log2scale * (A_s +- R_s)
    const int m = 10;
    std::vector<double> absA, AR, RA, RR, AA;
    for (int step = 0; step <= m; ++step) {
        double mx = 0.0;
        for (size_t i = 0; i < A.size(); ++i) mx = fmax(mx, fabs(A[i]) + R[i]);
        if (mx == 0.0) {
            *bound_out = 0.0;
            return EJOIN_OK;
        }
        int e;
        frexp(mx, &e);
        for (size_t i = 0; i < A.size(); ++i) {
            A[i] = ldexp(A[i], -e);
            R[i] = ldexp(R[i], -e);
        }
        log2scale += e;
        if (step == m) break;
        absA.resize(A.size());
        for (size_t i = 0; i < A.size(); ++i) absA[i] = fabs(A[i]);
        matmul(absA, R, AR, (int)k);
        matmul(R, absA, RA, (int)k);
        matmul(R, R, RR, (int)k);
        matmul(absA, absA, AA, (int)k);
        std::vector<double> A2;
        matmul(A, A, A2, (int)k);
        for (size_t i = 0; i < A.size(); ++i)
            R[i] = (AR[i] + RA[i] + RR[i] + gk * AA[i]) * marg;
        A.swap(A2);
        log2scale *= 2.0;
    }
    double fa = 0.0, fr = 0.0;
    for (size_t i = 0; i < A.size(); ++i) {
        fa += A[i] * A[i];
        fr += R[i] * R[i];
    }
    const double frob = (sqrt(fa) + sqrt(fr)) * (1.0 + 1e-12);
    // sigma_max = lambda_max(M)^(1/2) <= (2^log2scale * frob)^(1 / 2^(m+1))
    const double l2 = (log2(frob) + log2scale) / ldexp(1.0, m + 1);
    *bound_out = exp2(l2) * (1.0 + 1e-9);
    return EJOIN_OK;
}

}  // namespace ejoin

// ------------------------------------------------ projection files --
//
// A learned projection P (k x d FP32) with its certified spectral-norm bound,
// so that a trained P can be reused by later joins (ejoin_options.projection
// re-certifies it).  Little-endian layout:
//   0   8  magic "EJOINPRJ"
//   8   4  format version (1)
//   12  4  k
//   16  4  d
//   20  4  zero
//   24  8  sigma_cert (double)
//   32  4 k d  P, row-major FP32
//   ..  8  FNV-1a 64 of every byte before it
namespace {
constexpr char kProjMagic[8] = {'E', 'J', 'O', 'I', 'N', 'P', 'R', 'J'};
constexpr uint32_t kProjVersion = 1;

uint64_t fnv1a(const unsigned char* p, size_t n, uint64_t h = 1469598103934665603ull) {
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}
void put_u32(std::vector<unsigned char>& b, uint32_t v) {
    for (int i = 0; i < 4; ++i) b.push_back((unsigned char)(v >> (8 * i)));
}
void put_u64(std::vector<unsigned char>& b, uint64_t v) {
    for (int i = 0; i < 8; ++i) b.push_back((unsigned char)(v >> (8 * i)));
}
uint32_t get_u32(const unsigned char* p) {
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v |= (uint32_t)p[i] << (8 * i);
    return v;
}
uint64_t get_u64(const unsigned char* p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)p[i] << (8 * i);
    return v;
}
}  // namespace

int ejoin_save_projection(const char* filename, const float* P, uint32_t k, uint32_t d,
                          double sigma_cert) {
    ejoin::clear_error();
    if (!filename || !P || k == 0 || k > 16 || d == 0)
        return set_error(EJOIN_EINVAL, "bad arguments (k must be 1..16, d >= 1)");
    std::vector<unsigned char> b;
    b.insert(b.end(), kProjMagic, kProjMagic + 8);
    put_u32(b, kProjVersion);
    put_u32(b, k);
    put_u32(b, d);
    put_u32(b, 0);
    uint64_t sbits;
    memcpy(&sbits, &sigma_cert, 8);
    put_u64(b, sbits);
    for (uint64_t e = 0; e < (uint64_t)k * d; ++e) {
        uint32_t v;
        memcpy(&v, &P[e], 4);
        put_u32(b, v);
    }
    put_u64(b, fnv1a(b.data(), b.size()));
    FILE* f = fopen(filename, "wb");
    if (!f) return set_error(EJOIN_EIO, "could not open %s for writing", filename);
    const size_t w = fwrite(b.data(), 1, b.size(), f);
    const int c = fclose(f);
    if (w != b.size() || c != 0) return set_error(EJOIN_EIO, "short write on %s", filename);
    return EJOIN_OK;
}

int ejoin_load_projection(const char* filename, float* P_out, uint64_t capacity, uint32_t* k_out,
                          uint32_t* d_out, double* sigma_cert_out) {
    ejoin::clear_error();
    if (!filename) return set_error(EJOIN_EINVAL, "filename is NULL");
    std::vector<char> raw;
    if (!read_file(filename, raw)) return set_error(EJOIN_EIO, "could not open %s", filename);
    raw.pop_back();  // read_file's terminating NUL
    const unsigned char* p = reinterpret_cast<const unsigned char*>(raw.data());
    const size_t n = raw.size();
    if (n < 40 || memcmp(p, kProjMagic, 8) != 0)
        return set_error(EJOIN_EIO, "%s is not a projection file", filename);
    const uint32_t ver = get_u32(p + 8), k = get_u32(p + 12), d = get_u32(p + 16);
    if (ver != kProjVersion) return set_error(EJOIN_EIO, "%s: format version %u unsupported", filename, ver);
    if (k == 0 || k > 16 || d == 0 || n != 40 + 4ull * k * d)
        return set_error(EJOIN_EIO, "%s: bad header or size", filename);
    if (get_u64(p + n - 8) != fnv1a(p, n - 8))
        return set_error(EJOIN_EIO, "%s: checksum mismatch", filename);
    if (k_out) *k_out = k;
    if (d_out) *d_out = d;
    if (sigma_cert_out) {
        const uint64_t sbits = get_u64(p + 24);
        memcpy(sigma_cert_out, &sbits, 8);
    }
    if (P_out) {
        if (capacity < (uint64_t)k * d)
            return set_error(EJOIN_EINVAL, "P_out holds %llu of %u floats",
                             (unsigned long long)capacity, k * d);
        for (uint64_t e = 0; e < (uint64_t)k * d; ++e) {
            const uint32_t v = get_u32(p + 32 + 4 * e);
            memcpy(&P_out[e], &v, 4);
        }
    }
    return EJOIN_OK;
}
