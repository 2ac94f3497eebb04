/*
 * spike_gen.c -- seeded synthetic banded systems (libspike_gen.so).
 *
 * Produces A (0-based CSR, sorted columns), x_true and b = A x_true for the
 * synthetic workloads the solver is measured on.  Every random value is a
 * pure function of (seed, stream, index) through a splitmix64 hash, so the
 * output is identical whatever the thread count and on any host (no
 * floating-point in the hash; the only float step is the final scaling).
 *
 *   off-diagonal a_ij   ~ U[-1, 1)                     stream 0 (real), 3 (imag)
 *   diagonal a_ii       = dom * sum_j!=i |a_ij| * s_i  stream 1
 *                         s_i = +-1 (real) or e^{i theta}, theta ~ U[0, 2pi)
 *   x_true              ~ U[-1, 1)                     stream 2 (real), 4 (imag)
 *   b                   = A x_true, accumulated in double
 *
 * "Row |sum|" is read as the sum of |a_ij| over the off-diagonals present in
 * the row, which makes every row strictly diagonally dominant for dom > 1.
 * Complex data is interleaved {re, im} pairs (the C API's complex16).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

static inline uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* uniform in [-1, 1) from (seed, stream, idx) */
static inline double urand(uint64_t seed, uint64_t stream, uint64_t idx)
{
    uint64_t h = mix64(mix64(seed * 0x100000001B3ull + stream) ^ idx);
    return (double)(h >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

/* rowptr[n+1] for a full band (every in-range position within ku/kl). */
long long spike_gen_rowptr(int n, int ku, int kl, int *rowptr)
{
    long long nnz = 0;
    rowptr[0] = 0;
    for (int r = 0; r < n; r++) {
        int c0 = r - kl < 0 ? 0 : r - kl;
        int c1 = r + ku > n - 1 ? n - 1 : r + ku;
        nnz += c1 - c0 + 1;
        rowptr[r + 1] = (int)nnz;
    }
    return nnz;
}

/*
 * Fill colind/aij (aij: n_nnz doubles, or 2*n_nnz for complex), x_true and b
 * (n x nrhs column-major; doubled for complex).  rowptr must come from
 * spike_gen_rowptr with the same n, ku, kl.  Returns 0.
 */
int spike_gen_fill(int n, int ku, int kl, double dom, unsigned long long seed, int is_complex,
                   int nrhs, const int *rowptr, int *colind, double *aij, double *x_true, double *b)
{
    const int W = ku + kl + 1;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n; r++) {
        int c0 = r - kl < 0 ? 0 : r - kl;
        int c1 = r + ku > n - 1 ? n - 1 : r + ku;
        int t = rowptr[r];
        double offsum = 0.0;
        int tdiag = -1;
        for (int c = c0; c <= c1; c++, t++) {
            colind[t] = c;
            uint64_t idx = (uint64_t)r * (uint64_t)W + (uint64_t)(c - r + kl);
            if (c == r) {
                tdiag = t;
                continue;
            }
            if (is_complex) {
                double re = urand(seed, 0, idx), im = urand(seed, 3, idx);
                aij[2 * (size_t)t] = re;
                aij[2 * (size_t)t + 1] = im;
                offsum += sqrt(re * re + im * im);
            } else {
                double v = urand(seed, 0, idx);
                aij[t] = v;
                offsum += fabs(v);
            }
        }
        double mag = dom * offsum;
        if (mag == 0.0) mag = 1.0; /* a 1x1 system or an isolated row */
        if (is_complex) {
            double th = (urand(seed, 1, (uint64_t)r) + 1.0) * 3.14159265358979323846;
            aij[2 * (size_t)tdiag] = mag * cos(th);
            aij[2 * (size_t)tdiag + 1] = mag * sin(th);
        } else {
            aij[tdiag] = urand(seed, 1, (uint64_t)r) < 0.0 ? -mag : mag;
        }
    }
    const size_t N = (size_t)n;
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)N * nrhs; q++) {
        if (is_complex) {
            x_true[2 * q] = urand(seed, 2, (uint64_t)q);
            x_true[2 * q + 1] = urand(seed, 4, (uint64_t)q);
        } else {
            x_true[q] = urand(seed, 2, (uint64_t)q);
        }
    }
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n; r++) {
        for (int h = 0; h < nrhs; h++) {
            const size_t o = (size_t)h * N;
            double sr = 0.0, si = 0.0;
            for (int t = rowptr[r]; t < rowptr[r + 1]; t++) {
                size_t c = (size_t)colind[t];
                if (is_complex) {
                    double ar = aij[2 * (size_t)t], ai = aij[2 * (size_t)t + 1];
                    double xr = x_true[2 * (o + c)], xi = x_true[2 * (o + c) + 1];
                    sr += ar * xr - ai * xi;
                    si += ar * xi + ai * xr;
                } else {
                    sr += aij[t] * x_true[o + c];
                }
            }
            if (is_complex) {
                b[2 * (o + (size_t)r)] = sr;
                b[2 * (o + (size_t)r) + 1] = si;
            } else {
                b[o + (size_t)r] = sr;
            }
        }
    }
    return 0;
}
