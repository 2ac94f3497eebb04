/*
 * A host program written the way the reference's own drivers call the L1
 * plugin (OpenMP/spike_superlu.h:107-135) and the matrix helpers
 * (OpenMP/spike_matrix.h): it includes only the reference-named headers and
 * links against libspike_gb300.so.
 *
 *   compat_driver <matrix.bin> <nrhs> <max_nrhs>
 *
 * Loads the CSR file, solves A x = b for nrhs columns (b(:, j) = j + 1) twice
 * with one factorization, prints "ku kl relres" (max over columns of
 * ||b - A x|| / ||b||, computed here on the host) and exits 0 on success.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "spike_compat.h"

int main(int argc, char **argv)
{
    if (argc != 4) {
        fprintf(stderr, "usage: %s matrix.bin nrhs max_nrhs\n", argv[0]);
        return 2;
    }
    const int nrhs = atoi(argv[2]), max_nrhs = atoi(argv[3]);
    matrix_t *A = matrix_LoadCSR(argv[1]);
    if (!A) {
        fprintf(stderr, "%s\n", spike_last_error());
        return 1;
    }
    const int n = A->n;
    complex_t *b = malloc(sizeof(complex_t) * (size_t)n * nrhs);
    complex_t *x = calloc((size_t)n * nrhs, sizeof(complex_t));
    for (int j = 0; j < nrhs; j++)
        for (int i = 0; i < n; i++) b[(size_t)j * n + i] = j + 1.0;

    DirectSolverHander_t *h = directSolver_CreateHandler();
    if (!h || directSolver_Configure(h, max_nrhs) != SPIKE_SUCCESS ||
        directSolver_Factorize(h, n, (integer_t)A->nnz, A->colind, A->rowptr, A->aij) != SPIKE_SUCCESS) {
        fprintf(stderr, "%s\n", spike_last_error());
        return 1;
    }
    for (int pass = 0; pass < 2; pass++)
        if (directSolver_SolveForRHS(h, nrhs, x, b) != SPIKE_SUCCESS) {
            fprintf(stderr, "%s\n", spike_last_error());
            return 1;
        }
    directSolver_ShowStatistics(h);
    directSolver_Finalize(h);

    double worst = 0.0;
    for (int j = 0; j < nrhs; j++) {
        const complex_t *xj = x + (size_t)j * n, *bj = b + (size_t)j * n;
        double rr = 0.0, bb = 0.0;
        for (int r = 0; r < n; r++) {
            double s = bj[r];
            for (int t = A->rowptr[r]; t < A->rowptr[r + 1]; t++) s -= A->aij[t] * xj[A->colind[t]];
            rr += s * s;
            bb += bj[r] * bj[r];
        }
        const double rel = sqrt(rr) / sqrt(bb);
        if (rel > worst) worst = rel;
    }
    printf("%d %d %.6e\n", A->ku, A->kl, worst);
    matrix_Deallocate(A);
    free(x);
    free(b);
    return 0;
}
