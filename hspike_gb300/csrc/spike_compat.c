/*
 * spike_compat.c -- the reference's matrix helpers, CSR file format and
 * directSolver_* plugin (double build) on top of this library.  Host C only;
 * the plugin's factor and solve run on the GPU through spike_dfactor /
 * spike_dsolve_factored.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "spike_compat.h"
#include "spike_host_internal.h"

static double wall(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

Error_t matrix_ComputeBandwidth(const integer_t n, integer_t *colind, integer_t *rowptr, complex_t *aij,
                                integer_t *ku, integer_t *kl)
{
    (void)aij;
    if (n < 0 || !ku || !kl || (n > 0 && (!colind || !rowptr)))
        return spk_fail(SPIKE_ERR_ARGUMENT, "matrix_ComputeBandwidth: bad argument");
    int up = 0, lo = 0;
    for (int r = 0; r < n; r++)
        for (int t = rowptr[r]; t < rowptr[r + 1]; t++) {
            const int d = colind[t] - r;
            if (d > up) up = d;
            if (-d > lo) lo = -d;
        }
    *ku = up;
    *kl = lo;
    return spk_succeed();
}

matrix_t *matrix_LoadCSR(const char *filename)
{
    FILE *f = filename ? fopen(filename, "rb") : NULL;
    if (!f) {
        spk_fail(SPIKE_ERR_ARGUMENT, "matrix_LoadCSR: cannot open %s", filename ? filename : "(null)");
        return NULL;
    }
    integer_t hdr[3];
    matrix_t *M = NULL;
    if (fread(hdr, sizeof(integer_t), 3, f) != 3 || hdr[0] < 0 || hdr[1] < 0) {
        spk_fail(SPIKE_ERR_CSR, "matrix_LoadCSR: %s: bad header", filename);
        goto done;
    }
    if (hdr[2] != 0) {
        spk_fail(SPIKE_ERR_ARGUMENT, "matrix_LoadCSR: %s holds complex values (dtype flag %d); this is the real "
                 "build", filename, hdr[2]);
        goto done;
    }
    M = (matrix_t *)calloc(1, sizeof(matrix_t));
    if (!M) {
        spk_fail(SPIKE_ERR_MEMORY, "matrix_LoadCSR: host allocation failed");
        goto done;
    }
    M->n = hdr[0];
    M->nnz = (uLong_t)hdr[1];
    M->type = _DIAG_BLOCK_;
    M->aij = (complex_t *)malloc(sizeof(complex_t) * (M->nnz ? M->nnz : 1));
    M->colind = (integer_t *)malloc(sizeof(integer_t) * (M->nnz ? M->nnz : 1));
    M->rowptr = (integer_t *)malloc(sizeof(integer_t) * ((size_t)M->n + 1));
    if (!M->aij || !M->colind || !M->rowptr || fread(M->aij, sizeof(complex_t), M->nnz, f) != M->nnz ||
        fread(M->colind, sizeof(integer_t), M->nnz, f) != M->nnz ||
        fread(M->rowptr, sizeof(integer_t), (size_t)M->n + 1, f) != (size_t)M->n + 1) {
        matrix_Deallocate(M);
        M = NULL;
        spk_fail(SPIKE_ERR_CSR, "matrix_LoadCSR: %s: truncated file", filename);
        goto done;
    }
    matrix_ComputeBandwidth(M->n, M->colind, M->rowptr, M->aij, &M->ku, &M->kl);
    spk_succeed();
done:
    fclose(f);
    return M;
}

Error_t matrix_ExportBinary(matrix_t *M, const char *filename)
{
    if (!M || !filename) return spk_fail(SPIKE_ERR_ARGUMENT, "matrix_ExportBinary: NULL argument");
    FILE *f = fopen(filename, "wb");
    if (!f) return spk_fail(SPIKE_ERR_ARGUMENT, "matrix_ExportBinary: cannot open %s", filename);
    const integer_t hdr[3] = {M->n, (integer_t)M->nnz, 0};
    const int ok = fwrite(hdr, sizeof(integer_t), 3, f) == 3 &&
                   fwrite(M->aij, sizeof(complex_t), M->nnz, f) == M->nnz &&
                   fwrite(M->colind, sizeof(integer_t), M->nnz, f) == M->nnz &&
                   fwrite(M->rowptr, sizeof(integer_t), (size_t)M->n + 1, f) == (size_t)M->n + 1;
    if (fclose(f) != 0 || !ok) return spk_fail(SPIKE_ERR_ARGUMENT, "matrix_ExportBinary: write to %s failed", filename);
    return spk_succeed();
}

void matrix_SaveCSR(const char *filename, matrix_t *M) { matrix_ExportBinary(M, filename); }

matrix_t *matrix_CreateFromComponents(const integer_t n, const uLong_t nnz, integer_t *colind, integer_t *rowptr,
                                      complex_t *aij)
{
    matrix_t *A = (matrix_t *)calloc(1, sizeof(matrix_t));
    if (!A) {
        spk_fail(SPIKE_ERR_MEMORY, "matrix_CreateFromComponents: host allocation failed");
        return NULL;
    }
    A->n = n;
    A->nnz = nnz;
    A->colind = colind;
    A->rowptr = rowptr;
    A->aij = aij;
    A->type = _DIAG_BLOCK_;
    matrix_ComputeBandwidth(n, colind, rowptr, aij, &A->ku, &A->kl);
    return A;
}

Error_t matrix_Deallocate(matrix_t *M)
{
    if (!M) return spk_fail(SPIKE_ERR_ARGUMENT, "matrix_Deallocate: NULL matrix");
    free(M->colind);
    free(M->rowptr);
    free(M->aij);
    free(M);
    return spk_succeed();
}

block_t *block_CreateEmptyBlock(const integer_t n, const integer_t m, const integer_t ku, const integer_t kl,
                                blocktype_t type, blocksection_t section)
{
    if (n < 0 || m < 0) {
        spk_fail(SPIKE_ERR_ARGUMENT, "block_CreateEmptyBlock: negative size %d x %d", n, m);
        return NULL;
    }
    const size_t count = (size_t)n * (size_t)m;
    block_t *B = (block_t *)calloc(1, sizeof(block_t));
    complex_t *a = (complex_t *)calloc(count ? count : 1, sizeof(complex_t));
    if (!B || !a) {
        free(B);
        free(a);
        spk_fail(SPIKE_ERR_MEMORY, "block_CreateEmptyBlock: host allocation failed");
        return NULL;
    }
    B->type = type;
    B->section = section;
    B->n = n;
    B->m = m;
    B->ku = ku;
    B->kl = kl;
    B->aij = a;
    spk_succeed();
    return B;
}

Error_t block_Deallocate(block_t *B)
{
    if (!B) return spk_fail(SPIKE_ERR_ARGUMENT, "block_Deallocate: NULL block");
    free(B->aij);
    free(B);
    return spk_succeed();
}

void block_SaveCSR(const char *filename, block_t *B)
{
    if (!B || !filename) {
        spk_fail(SPIKE_ERR_ARGUMENT, "block_SaveCSR: NULL argument");
        return;
    }
    FILE *f = fopen(filename, "wb");
    if (!f) {
        spk_fail(SPIKE_ERR_ARGUMENT, "block_SaveCSR: cannot open %s", filename);
        return;
    }
    const integer_t hdr[6] = {(integer_t)B->type, (integer_t)B->section, B->n, B->m, B->ku, B->kl};
    const size_t count = (size_t)B->n * (size_t)B->m;
    const int ok = fwrite(hdr, sizeof(integer_t), 6, f) == 6 && fwrite(B->aij, sizeof(complex_t), count, f) == count;
    if (fclose(f) != 0 || !ok)
        spk_fail(SPIKE_ERR_ARGUMENT, "block_SaveCSR: write to %s failed", filename);
    else
        spk_succeed();
}

block_t *block_loadCSR(const char *filename)
{
    FILE *f = filename ? fopen(filename, "rb") : NULL;
    if (!f) {
        spk_fail(SPIKE_ERR_ARGUMENT, "block_loadCSR: cannot open %s", filename ? filename : "(null)");
        return NULL;
    }
    integer_t hdr[6];
    block_t *B = NULL;
    if (fread(hdr, sizeof(integer_t), 6, f) != 6 || hdr[2] < 0 || hdr[3] < 0) {
        spk_fail(SPIKE_ERR_CSR, "block_loadCSR: %s: bad header", filename);
    } else if ((B = block_CreateEmptyBlock(hdr[2], hdr[3], hdr[4], hdr[5], (blocktype_t)hdr[0],
                                           (blocksection_t)hdr[1])) != NULL) {
        const size_t count = (size_t)B->n * (size_t)B->m;
        if (fread(B->aij, sizeof(complex_t), count, f) != count) {
            block_Deallocate(B);
            B = NULL;
            spk_fail(SPIKE_ERR_CSR, "block_loadCSR: %s: truncated file", filename);
        }
    }
    fclose(f);
    return B;
}

/* n raw elements of the given size, or NULL */
static void *load_raw(const integer_t n, const char *filename, size_t elem, const char *who)
{
    if (n < 0 || !filename) {
        spk_fail(SPIKE_ERR_ARGUMENT, "%s: bad argument", who);
        return NULL;
    }
    FILE *f = fopen(filename, "rb");
    if (!f) {
        spk_fail(SPIKE_ERR_ARGUMENT, "%s: cannot open %s", who, filename);
        return NULL;
    }
    void *p = malloc(elem * (n ? (size_t)n : 1));
    if (!p)
        spk_fail(SPIKE_ERR_MEMORY, "%s: host allocation failed", who);
    else if (fread(p, elem, (size_t)n, f) != (size_t)n) {
        free(p);
        p = NULL;
        spk_fail(SPIKE_ERR_ARGUMENT, "%s: %s holds fewer than %d entries", who, filename, n);
    } else
        spk_succeed();
    fclose(f);
    return p;
}

integer_t *vector_LoadPermutationArray(const integer_t n, const char *filename)
{
    return (integer_t *)load_raw(n, filename, sizeof(integer_t), "vector_LoadPermutationArray");
}

complex_t *vector_LoadRHS(const integer_t n, const char *filename)
{
    return (complex_t *)load_raw(n, filename, sizeof(complex_t), "vector_LoadRHS");
}

/* ------------------------------------------------------------------ */
/* inner-solver plugin                                                  */
/* ------------------------------------------------------------------ */
DirectSolverHander_t *directSolver_CreateHandler(void)
{
    DirectSolverHander_t *h = (DirectSolverHander_t *)calloc(1, sizeof *h);
    if (!h) {
        spk_fail(SPIKE_ERR_MEMORY, "directSolver_CreateHandler: host allocation failed");
        return NULL;
    }
    if (spike_context_create(&h->ctx) != SPIKE_SUCCESS) {
        free(h);
        return NULL; /* detail (e.g. no device) left by spike_context_create */
    }
    h->max_nrhs = RHS_CHUNK;
    return h;
}

Error_t directSolver_Configure(DirectSolverHander_t *h, const integer_t max_nrhs)
{
    if (!h || max_nrhs < 1) return spk_fail(SPIKE_ERR_ARGUMENT, "directSolver_Configure: bad argument");
    h->max_nrhs = max_nrhs;
    return spk_succeed();
}

Error_t directSolver_Factorize(DirectSolverHander_t *h, const integer_t n, const integer_t nnz, integer_t *colind,
                               integer_t *rowptr, complex_t *aij)
{
    if (!h) return spk_fail(SPIKE_ERR_HANDLE, "directSolver_Factorize: NULL handler");
    if (h->factor) {
        spike_factor_release(h->factor);
        h->factor = NULL;
    }
    const double t0 = wall();
    const Error_t rc = spike_dfactor(h->ctx, n, nnz, colind, rowptr, aij, &h->factor);
    h->factor_t += wall() - t0;
    if (rc == SPIKE_SUCCESS) h->n = n;
    return rc;
}

Error_t directSolver_SolveForRHS(DirectSolverHander_t *h, const integer_t nrhs, complex_t *xij, complex_t *bij)
{
    if (!h || !h->factor) return spk_fail(SPIKE_ERR_HANDLE, "directSolver_SolveForRHS: no factorization");
    if (nrhs < 0) return spk_fail(SPIKE_ERR_ARGUMENT, "directSolver_SolveForRHS: nrhs must be >= 0");
    const double t0 = wall();
    Error_t rc = SPIKE_SUCCESS;
    for (int h0 = 0; h0 < nrhs && rc == SPIKE_SUCCESS; h0 += h->max_nrhs) {
        const int nr = nrhs - h0 < h->max_nrhs ? nrhs - h0 : h->max_nrhs;
        rc = spike_dsolve_factored(h->factor, nr, xij + (size_t)h0 * h->n, bij + (size_t)h0 * h->n);
        h->rhs_block_count++;
        h->rhs_column_count += nr;
    }
    h->solve_t += wall() - t0;
    return rc == SPIKE_SUCCESS ? spk_succeed() : rc;
}

Error_t directSolver_ShowStatistics(DirectSolverHander_t *h)
{
    if (!h) return spk_fail(SPIKE_ERR_HANDLE, "directSolver_ShowStatistics: NULL handler");
    fprintf(stderr, "directSolver (GB300): factor %.6f s, solve %.6f s, %d right-hand-side blocks, %d columns\n",
            h->factor_t, h->solve_t, h->rhs_block_count, h->rhs_column_count);
    return spk_succeed();
}

Error_t directSolver_Finalize(DirectSolverHander_t *h)
{
    if (!h) return spk_fail(SPIKE_ERR_HANDLE, "directSolver_Finalize: NULL handler");
    if (h->factor) spike_factor_release(h->factor);
    spike_context_destroy(h->ctx);
    free(h);
    return spk_succeed();
}

Error_t directSolver_Solve(integer_t n, integer_t nnz, integer_t nrhs, integer_t *colind, integer_t *rowptr,
                           complex_t *aij, complex_t *xij, complex_t *bij)
{
    DirectSolverHander_t *h = directSolver_CreateHandler();
    if (!h) return SPIKE_ERROR;
    Error_t rc = directSolver_Factorize(h, n, nnz, colind, rowptr, aij);
    if (rc == SPIKE_SUCCESS) rc = directSolver_SolveForRHS(h, nrhs, xij, bij);
    /* keep the first failure's detail */
    char msg[512];
    const int code = spike_last_error_code();
    snprintf(msg, sizeof msg, "%s", spike_last_error());
    directSolver_Finalize(h);
    if (rc != SPIKE_SUCCESS) return spk_fail(code, "%s", msg);
    return spk_succeed();
}
