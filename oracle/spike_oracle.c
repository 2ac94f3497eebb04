/*
 * spike_oracle.c -- CPU restatement of the reference SPIKE solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU path is
 * compared against; the product library never links, loads or calls it.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * it.
 *
 * It follows the reference's shared-memory solve, OpenMP/spike_interfaces.c
 * :43-419, step by step:
 *   - bandwidth as in matrix_ComputeBandwidth  (OpenMP/spike_algebra.c:56-95)
 *   - schedule as in spike_solve_analysis       (OpenMP/spike_analysis.c:38-76)
 *   - the reduced system R as a CSR matrix with exactly the reference's
 *     row/column layout: matrix_CreateEmptyReducedSystem
 *     (OpenMP/spike_matrix.c:657-740) and matrix_AddTipToReducedMatrix
 *     (OpenMP/spike_matrix.c:1414-1495); the reduced RHS as in
 *     block_AddTipTOReducedRHS (OpenMP/spike_matrix.c:1272-1297)
 *   - tips: top = first ku rows, bottom = last kl rows
 *     (block_ExtractTip, OpenMP/spike_matrix.c:1013-1057)
 *   - implicit retrieval x_i = A_i^{-1}(f_i - B_i x_t - C_i x_b)
 *     (OpenMP/spike_interfaces.c:259-396)
 * The inner solver is a banded LU with partial pivoting written from the
 * textbook algorithm (the reference uses SuperLU_MT pdgstrf with partial
 * pivoting, OpenMP/spike_superlu.c:763); the reduced system, which the
 * reference hands to MKL PARDISO (OpenMP/spike_algebra.c:263-420), is solved
 * with the same banded LU on R's own band.  The reference's nrhs>1 retrieval
 * defect (OpenMP/spike_matrix.c:1341-1342) is not reproduced: every column of
 * x is written.
 *
 * Compiled twice: once as real double (prefix d) and once with
 * -DORACLE_COMPLEX as double complex (prefix z).  Partitions are processed in
 * parallel with OpenMP when it is enabled (the reference loops serially).
 */
#include <complex.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORACLE_COMPLEX
typedef double complex scalar;
#define PFX(name) z##name
#define SABS(v) cabs(v)
#else
typedef double scalar;
#define PFX(name) d##name
#define SABS(v) fabs(v)
#endif

/* ------------------------------------------------------------------ */
/* type-independent helpers (built once, in the real translation unit) */
/* ------------------------------------------------------------------ */
#ifndef ORACLE_COMPLEX
/* matrix_ComputeBandwidth, OpenMP/spike_algebra.c:56-95:
 * ku = max(col - row), kl = max(row - col), both >= 0. */
int oracle_bandwidth(int n, const int *rowptr, const int *colind, int *ku, int *kl)
{
    int u = 0, l = 0;
    for (int r = 0; r < n; r++)
        for (int t = rowptr[r]; t < rowptr[r + 1]; t++) {
            int c = colind[t];
            if (c - r > u) u = c - r;
            if (r - c > l) l = r - c;
        }
    *ku = u;
    *kl = l;
    return 0;
}

/* spike_solve_analysis, OpenMP/spike_analysis.c:38-76: regular partitions of
 * floor(n/p) rows, the remainder in the last one; reduced-system row offsets
 * r[i+1] = r[i] + ku + kl. */
int oracle_schedule(int n, int p, int ku, int kl, int *nb, int *rb)
{
    if (p < 1 || n < p) return 1;
    int nreg = n / p;
    nb[0] = 0;
    rb[0] = 0;
    for (int i = 1; i < p; i++) {
        nb[i] = i * nreg;
        rb[i] = rb[i - 1] + ku + kl;
    }
    nb[p] = n;
    rb[p] = rb[p - 1] + ku + kl;
    return 0;
}

/* GetNnzAndRowsUpToPartition, OpenMP/spike_matrix.c:1379-1412 (ku, kl equal
 * in every partition, as the reference's schedule makes them). */
int64_t oracle_reduced_nnz_before(int P, int part, int ku, int kl)
{
    int64_t nnz = 0;
    for (int q = 0; q < part; q++) {
        if (q == 0)
            nnz = (int64_t)ku * (ku + kl);
        else if (q == P - 1)
            nnz += (int64_t)kl * (ku + kl);
        else
            nnz += (int64_t)kl * (ku + kl) + (int64_t)ku * (ku + kl);
        nnz += ku + kl;
    }
    return nnz;
}

int64_t oracle_reduced_nnz(int P, int ku, int kl)
{
    return oracle_reduced_nnz_before(P, P, ku, kl);
}

/* Pattern of R, matrix_CreateEmptyReducedSystem (OpenMP/spike_matrix.c
 * :657-740): each row holds [W-tip columns of the previous partition's bottom]
 * [its own diagonal] [V-tip columns of the next partition's top]. */
int oracle_reduced_pattern(int P, int ku, int kl, int *rowptr, int *colind)
{
    int nrows = P * (ku + kl);
    int64_t nnz = 0;
    rowptr[0] = 0;
    for (int q = 0; q < P; q++) {
        int r0 = q * (ku + kl), r1 = (q + 1) * (ku + kl);
        for (int row = r0; row < r1; row++) {
            if (q > 0)
                for (int c = r0 - kl; c < r0; c++) colind[nnz++] = c;
            colind[nnz++] = row;
            if (q < P - 1)
                for (int c = r1; c < r1 + ku; c++) colind[nnz++] = c;
            rowptr[row + 1] = (int)nnz;
        }
    }
    (void)nrows;
    return 0;
}

/* Threads for the partition loops of later calls (0: the OpenMP default);
 * returns the previous limit.  Used to time the oracle on one core. */
int oracle_set_threads(int threads)
{
#ifdef _OPENMP
    const int prev = omp_get_max_threads();
    static int dflt = 0;
    if (!dflt) dflt = prev;
    omp_set_num_threads(threads > 0 ? threads : dflt);
    return prev;
#else
    (void)threads;
    return 1;
#endif
}
#endif /* !ORACLE_COMPLEX */

int oracle_bandwidth(int n, const int *rowptr, const int *colind, int *ku, int *kl);
int oracle_schedule(int n, int p, int ku, int kl, int *nb, int *rb);
int64_t oracle_reduced_nnz(int P, int ku, int kl);
int64_t oracle_reduced_nnz_before(int P, int part, int ku, int kl);
int oracle_reduced_pattern(int P, int ku, int kl, int *rowptr, int *colind);

/* ------------------------------------------------------------------ */
/* banded LU with partial pivoting                                     */
/* ------------------------------------------------------------------ */
/* Storage: column-major band with ld = 2*kl + ku + 1; element (i, j) of the
 * m x m matrix lives at ab[(kl + ku + i - j) + j*ld] for
 * j - (ku + kl) <= i <= j + kl.  The top kl rows hold U's fill from row
 * interchanges. */
typedef struct {
    int m, kl, ku, ld;
    scalar *ab;
    int *piv;
} band_lu;

#define AB(F, i, j) ((F)->ab[(size_t)((F)->kl + (F)->ku + (i) - (j)) + (size_t)(j) * (F)->ld])

static int band_alloc(band_lu *F, int m, int kl, int ku)
{
    F->m = m;
    F->kl = kl;
    F->ku = ku;
    F->ld = 2 * kl + ku + 1;
    F->ab = (scalar *)calloc((size_t)F->ld * (size_t)m, sizeof(scalar));
    F->piv = (int *)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    return (F->ab && F->piv) ? 0 : 1;
}

static void band_free(band_lu *F)
{
    free(F->ab);
    free(F->piv);
    F->ab = NULL;
    F->piv = NULL;
}

/* Gaussian elimination with row partial pivoting restricted to the band.
 * Returns 0, or j+1 if column j has an exactly zero pivot. */
static int band_factor(band_lu *F)
{
    const int m = F->m, kl = F->kl, ku = F->ku;
    int ju = 0; /* last column touched by U so far */
    for (int j = 0; j < m; j++) {
        int km = kl < m - 1 - j ? kl : m - 1 - j;
        int jp = 0;
        double best = SABS(AB(F, j, j));
        for (int i = 1; i <= km; i++) {
            double v = SABS(AB(F, j + i, j));
            if (v > best) {
                best = v;
                jp = i;
            }
        }
        F->piv[j] = j + jp;
        if (best == 0.0) return j + 1;
        int jend = j + ku + jp;
        if (jend > m - 1) jend = m - 1;
        if (jend > ju) ju = jend;
        if (jp != 0)
            for (int c = j; c <= ju; c++) {
                scalar t = AB(F, j, c);
                AB(F, j, c) = AB(F, j + jp, c);
                AB(F, j + jp, c) = t;
            }
        scalar inv = 1.0 / AB(F, j, j);
        for (int i = 1; i <= km; i++) AB(F, j + i, j) *= inv;
        for (int c = j + 1; c <= ju; c++) {
            scalar u = AB(F, j, c);
            if (u != 0.0)
                for (int i = 1; i <= km; i++) AB(F, j + i, c) -= AB(F, j + i, j) * u;
        }
    }
    return 0;
}

/* Solve with the factors for nrhs columns of b (column-major, ld = ldb). */
static void band_solve(const band_lu *F, int nrhs, scalar *b, int ldb)
{
    const int m = F->m, kl = F->kl, ku = F->ku;
    for (int c = 0; c < nrhs; c++) {
        scalar *x = b + (size_t)c * ldb;
        for (int j = 0; j < m; j++) {
            int km = kl < m - 1 - j ? kl : m - 1 - j;
            int p = F->piv[j];
            if (p != j) {
                scalar t = x[j];
                x[j] = x[p];
                x[p] = t;
            }
            scalar v = x[j];
            if (v != 0.0)
                for (int i = 1; i <= km; i++) x[j + i] -= AB(F, j + i, j) * v;
        }
        for (int j = m - 1; j >= 0; j--) {
            x[j] /= AB(F, j, j);
            scalar v = x[j];
            int i0 = j - (ku + kl);
            if (i0 < 0) i0 = 0;
            if (v != 0.0)
                for (int i = i0; i < j; i++) x[i] -= AB(F, i, j) * v;
        }
    }
}

/* matrix_ExtractMatrix (OpenMP/spike_matrix.c:563-645) followed by the
 * factorization: rows [r0, r1) x columns [r0, r1) of A into band storage. */
static int factor_block(band_lu *F, const int *rowptr, const int *colind, const scalar *aij,
                        int r0, int r1, int kl, int ku)
{
    int m = r1 - r0;
    if (band_alloc(F, m, kl, ku)) return -1;
    for (int r = r0; r < r1; r++)
        for (int t = rowptr[r]; t < rowptr[r + 1]; t++) {
            int c = colind[t];
            if (c >= r0 && c < r1) AB(F, r - r0, c - r0) = aij[t];
        }
    return band_factor(F);
}

/* ------------------------------------------------------------------ */
/* the SPIKE solve                                                     */
/* ------------------------------------------------------------------ */
/*
 * PFX(oracle_spike): x = A^{-1} b with P partitions.
 *
 * Optional outputs (pass NULL to skip):
 *   R_rowptr[P*(ku+kl)+1], R_colind[nnzR], R_aij[nnzR]: the reduced system;
 *   xr[P*(ku+kl) x nrhs]: its right-hand side; yr: its solution.
 * Returns 0 on success, 2 for a bad schedule, 3 for a singular block,
 * 4 for a singular reduced system, -1 on allocation failure.
 */
int PFX(oracle_spike)(int n, int nnz, int nrhs, const int *colind, const int *rowptr,
                      const scalar *aij, scalar *x, const scalar *b, int P,
                      int *R_rowptr, int *R_colind, scalar *R_aij, scalar *xr_out,
                      scalar *yr_out)
{
    (void)nnz;
    int ku, kl;
    oracle_bandwidth(n, rowptr, colind, &ku, &kl);
    if (P < 1) P = 4; /* compute_optimal_number_of_partitions returns 4 */
    int *nb = (int *)malloc(sizeof(int) * (P + 1));
    int *rb = (int *)malloc(sizeof(int) * (P + 1));
    if (oracle_schedule(n, P, ku, kl, nb, rb)) {
        free(nb);
        free(rb);
        return 2;
    }

    if (P == 1) { /* no coupling: a single direct solve */
        band_lu F;
        int st = factor_block(&F, rowptr, colind, aij, 0, n, kl, ku);
        if (st == 0) {
            memcpy(x, b, sizeof(scalar) * (size_t)n * nrhs);
            band_solve(&F, nrhs, x, n);
        }
        band_free(&F);
        free(nb);
        free(rb);
        return st == 0 ? 0 : (st < 0 ? -1 : 3);
    }

    const int nR = rb[P];
    const int64_t nnzR = oracle_reduced_nnz(P, ku, kl);
    int *Rp = (int *)malloc(sizeof(int) * (nR + 1));
    int *Rc = (int *)malloc(sizeof(int) * (size_t)(nnzR > 0 ? nnzR : 1));
    scalar *Ra = (scalar *)calloc((size_t)(nnzR > 0 ? nnzR : 1), sizeof(scalar));
    scalar *xr = (scalar *)calloc((size_t)nR * nrhs, sizeof(scalar));
    band_lu *Fs = (band_lu *)calloc((size_t)P, sizeof(band_lu));
    int status = 0;
    oracle_reduced_pattern(P, ku, kl, Rp, Rc);
    /* the diagonal entries of R are one (spike_matrix.c:692-693) */
    for (int row = 0; row < nR; row++)
        for (int t = Rp[row]; t < Rp[row + 1]; t++)
            if (Rc[t] == row) Ra[t] = 1.0;

    /* ---- factorization phase (spike_interfaces.c:105-237) ---- */
#pragma omp parallel for schedule(dynamic, 1) reduction(max : status)
    for (int q = 0; q < P; q++) {
        const int r0 = nb[q], r1 = nb[q + 1], m = r1 - r0;
        band_lu *F = &Fs[q];
        int st = factor_block(F, rowptr, colind, aij, r0, r1, kl, ku);
        if (st != 0) {
            status = st < 0 ? 1 : 3;
            continue;
        }
        /* y_i = A_i^{-1} f_i and its tips into the reduced RHS */
        scalar *y = (scalar *)malloc(sizeof(scalar) * (size_t)m * nrhs);
        for (int c = 0; c < nrhs; c++)
            memcpy(y + (size_t)c * m, b + (size_t)c * n + r0, sizeof(scalar) * m);
        band_solve(F, nrhs, y, m);
        for (int c = 0; c < nrhs; c++) {
            for (int t = 0; t < ku; t++) xr[(size_t)c * nR + rb[q] + t] = y[(size_t)c * m + t];
            for (int t = 0; t < kl; t++)
                xr[(size_t)c * nR + rb[q] + ku + t] = y[(size_t)c * m + m - kl + t];
        }
        free(y);

        /* row-major running index into this partition's R entries, walking the
         * rows exactly as matrix_AddTipToReducedMatrix does */
        int64_t base = oracle_reduced_nnz_before(P, q, ku, kl);
        int wcols = q > 0 ? kl : 0, vcols = q < P - 1 ? ku : 0;
        int rowlen = wcols + 1 + vcols;
        if (q < P - 1) { /* V_i = A_i^{-1} B_i, B_i = A[r0:r1, r1:r1+ku] */
            scalar *V = (scalar *)calloc((size_t)m * ku, sizeof(scalar));
            for (int r = r0; r < r1; r++)
                for (int t = rowptr[r]; t < rowptr[r + 1]; t++) {
                    int c = colind[t];
                    if (c >= r1 && c < r1 + ku) V[(size_t)(c - r1) * m + (r - r0)] = aij[t];
                }
            band_solve(F, ku, V, m);
            for (int t = 0; t < ku + kl; t++) {
                int vr = t < ku ? t : m - kl + (t - ku); /* top ku rows, bottom kl */
                for (int c = 0; c < ku; c++)
                    Ra[base + (int64_t)t * rowlen + wcols + 1 + c] = V[(size_t)c * m + vr];
            }
            free(V);
        }
        if (q > 0) { /* W_i = A_i^{-1} C_i, C_i = A[r0:r1, r0-kl:r0] */
            scalar *W = (scalar *)calloc((size_t)m * kl, sizeof(scalar));
            for (int r = r0; r < r1; r++)
                for (int t = rowptr[r]; t < rowptr[r + 1]; t++) {
                    int c = colind[t];
                    if (c >= r0 - kl && c < r0) W[(size_t)(c - (r0 - kl)) * m + (r - r0)] = aij[t];
                }
            band_solve(F, kl, W, m);
            for (int t = 0; t < ku + kl; t++) {
                int wr = t < ku ? t : m - kl + (t - ku);
                for (int c = 0; c < kl; c++)
                    Ra[base + (int64_t)t * rowlen + c] = W[(size_t)c * m + wr];
            }
            free(W);
        }
    }

    /* ---- reduced system (spike_interfaces.c:243-245) ---- */
    scalar *yr = (scalar *)malloc(sizeof(scalar) * (size_t)nR * nrhs);
    if (status == 0) {
        int rku, rkl;
        oracle_bandwidth(nR, Rp, Rc, &rku, &rkl);
        band_lu FR;
        if (band_alloc(&FR, nR, rkl, rku)) {
            status = 1;
        } else {
            for (int row = 0; row < nR; row++)
                for (int t = Rp[row]; t < Rp[row + 1]; t++) AB(&FR, row, Rc[t]) = Ra[t];
            if (band_factor(&FR) != 0) {
                status = 4;
            } else {
                memcpy(yr, xr, sizeof(scalar) * (size_t)nR * nrhs);
                band_solve(&FR, nrhs, yr, nR);
            }
            band_free(&FR);
        }
    }

    /* ---- retrieval (spike_interfaces.c:259-396) ---- */
    if (status == 0) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int q = 0; q < P; q++) {
            const int r0 = nb[q], r1 = nb[q + 1], m = r1 - r0;
            scalar *f = (scalar *)malloc(sizeof(scalar) * (size_t)m * nrhs);
            for (int c = 0; c < nrhs; c++)
                memcpy(f + (size_t)c * m, b + (size_t)c * n + r0, sizeof(scalar) * m);
            if (q < P - 1) { /* f[m-ku:m] -= B_i x_t(next): rows r1-ku..r1, cols r1..r1+ku */
                for (int r = r1 - ku; r < r1; r++)
                    for (int t = rowptr[r]; t < rowptr[r + 1]; t++) {
                        int c = colind[t];
                        if (c >= r1 && c < r1 + ku)
                            for (int h = 0; h < nrhs; h++)
                                f[(size_t)h * m + (r - r0)] -= aij[t] * yr[(size_t)h * nR + rb[q + 1] + (c - r1)];
                    }
            }
            if (q > 0) { /* f[0:kl] -= C_i x_b(prev): rows r0..r0+kl, cols r0-kl..r0 */
                for (int r = r0; r < r0 + kl; r++)
                    for (int t = rowptr[r]; t < rowptr[r + 1]; t++) {
                        int c = colind[t];
                        if (c >= r0 - kl && c < r0)
                            for (int h = 0; h < nrhs; h++)
                                f[(size_t)h * m + (r - r0)] -= aij[t] * yr[(size_t)h * nR + rb[q] - kl + (c - (r0 - kl))];
                    }
            }
            band_solve(&Fs[q], nrhs, f, m);
            for (int h = 0; h < nrhs; h++)
                memcpy(x + (size_t)h * n + r0, f + (size_t)h * m, sizeof(scalar) * m);
            free(f);
        }
    }

    if (R_rowptr) memcpy(R_rowptr, Rp, sizeof(int) * (nR + 1));
    if (R_colind) memcpy(R_colind, Rc, sizeof(int) * (size_t)nnzR);
    if (R_aij) memcpy(R_aij, Ra, sizeof(scalar) * (size_t)nnzR);
    if (xr_out) memcpy(xr_out, xr, sizeof(scalar) * (size_t)nR * nrhs);
    if (yr_out && status == 0) memcpy(yr_out, yr, sizeof(scalar) * (size_t)nR * nrhs);

    for (int q = 0; q < P; q++) band_free(&Fs[q]);
    free(Fs);
    free(yr);
    free(xr);
    free(Ra);
    free(Rc);
    free(Rp);
    free(nb);
    free(rb);
    return status;
}

/* Direct banded solve of the whole system: the FP64 error oracle. */
int PFX(oracle_direct)(int n, int nrhs, const int *colind, const int *rowptr, const scalar *aij,
                       scalar *x, const scalar *b)
{
    int ku, kl;
    oracle_bandwidth(n, rowptr, colind, &ku, &kl);
    band_lu F;
    int st = factor_block(&F, rowptr, colind, aij, 0, n, kl, ku);
    if (st == 0) {
        memcpy(x, b, sizeof(scalar) * (size_t)n * nrhs);
        band_solve(&F, nrhs, x, n);
    }
    band_free(&F);
    return st == 0 ? 0 : (st < 0 ? -1 : 3);
}

/* r = b - A x per column, and ||r||_2 / ||b||_2 per column
 * (ComputeResidualOfLinearSystem, OpenMP/spike_algebra.c:97-151, for every
 * column instead of the first five). */
void PFX(oracle_residual)(int n, int nrhs, const int *colind, const int *rowptr, const scalar *aij,
                          const scalar *x, const scalar *b, double *relres)
{
    for (int h = 0; h < nrhs; h++) {
        double rr = 0.0, bb = 0.0;
        const scalar *xh = x + (size_t)h * n, *bh = b + (size_t)h * n;
        for (int r = 0; r < n; r++) {
            scalar s = bh[r];
            for (int t = rowptr[r]; t < rowptr[r + 1]; t++) s -= aij[t] * xh[colind[t]];
            double a = SABS(s), c = SABS(bh[r]);
            rr += a * a;
            bb += c * c;
        }
        relres[h] = bb > 0.0 ? sqrt(rr) / sqrt(bb) : sqrt(rr);
    }
}
