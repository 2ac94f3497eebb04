/*
 * spike_compat.h -- the reference's matrix types, CSR file format and
 * inner-solver plugin interface, for code written against the reference's
 * double build (compiled with -D_DATATYPE_D_), so that it links unchanged.
 *
 *   types        matrix_t / block_t and their enums (OpenMP/spike_matrix.h:34-72)
 *   bandwidth    matrix_ComputeBandwidth (OpenMP/spike_algebra.c:56-95)
 *   CSR files    matrix_LoadCSR / matrix_SaveCSR / matrix_ExportBinary
 *                (OpenMP/spike_matrix.c:11-214): int32 n, int32 nnz, int32
 *                dtype flag, nnz values, int32 colind[nnz], int32 rowptr[n+1]
 *   wrapping     matrix_CreateFromComponents / matrix_Deallocate
 *                (OpenMP/spike_matrix.c:243-272)
 *   blocks       block_CreateEmptyBlock / block_Deallocate
 *                (OpenMP/spike_matrix.c:746-776,910-916); block files
 *                block_SaveCSR / block_loadCSR (OpenMP/spike_matrix.c:90-153):
 *                int32 type, section, n, m, ku, kl, then n*m values
 *                column-major
 *   vectors      vector_LoadPermutationArray / vector_LoadRHS
 *                (OpenMP/spike_matrix.c:155-179): n raw int32 / n raw values
 *   plugin       directSolver_* (OpenMP/spike_superlu.h:107-135): factor once,
 *                solve many, here on the GPU through the factor handles of
 *                spike_gb300.h instead of SuperLU_MT
 *
 * Differences from the reference: errors return NULL / SPIKE_ERROR with the
 * detail in spike_last_error() instead of aborting; matrix_LoadCSR reads the
 * dtype flag (0 = real) and refuses a complex file (flag 1, planar) rather
 * than misreading it; matrix_SaveCSR writes the flag 0 (the reference writes
 * M->type there, OpenMP/spike_matrix.c:71).
 */
#ifndef SPIKE_COMPAT_H
#define SPIKE_COMPAT_H

#include "spike_datatypes.h"
#include "spike_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef double complex_t; /* the reference's scalar type in its double build */

typedef enum { _C_BLOCK_, _DIAG_BLOCK_, _B_BLOCK_ } matrixtype_t;

typedef struct {
    integer_t n;
    uLong_t nnz;
    integer_t ku;
    integer_t kl;
    matrixtype_t type;
    integer_t *colind;
    integer_t *rowptr;
    complex_t *aij;
} matrix_t;

typedef enum { _V_BLOCK_, _W_BLOCK_, _RHS_BLOCK_ } blocktype_t;
typedef enum { _TOP_SECTION_, _CENTRAL_SECTION_, _BOTTOM_SECTION_, _WHOLE_SECTION_ } blocksection_t;

typedef struct {
    blocktype_t type;
    blocksection_t section;
    integer_t n;
    integer_t m;
    integer_t ku;
    integer_t kl;
    complex_t *aij;
} block_t;

/* ku = max(col - row), kl = max(row - col) over the stored entries (host). */
Error_t matrix_ComputeBandwidth(const integer_t n, integer_t *colind, integer_t *rowptr, complex_t *aij,
                                integer_t *ku, integer_t *kl);
/* Read a CSR file (real values); NULL on error.  Free with matrix_Deallocate. */
matrix_t *matrix_LoadCSR(const char *filename);
/* Write M in the same format (dtype flag 0). */
void matrix_SaveCSR(const char *filename, matrix_t *M);
Error_t matrix_ExportBinary(matrix_t *M, const char *filename);
/* Wrap caller arrays (not copied; matrix_Deallocate frees them with free()),
 * bandwidth computed. */
matrix_t *matrix_CreateFromComponents(const integer_t n, const uLong_t nnz, integer_t *colind, integer_t *rowptr,
                                      complex_t *aij);
Error_t matrix_Deallocate(matrix_t *M);

/* n x m zero block (column-major); NULL on a negative size. */
block_t *block_CreateEmptyBlock(const integer_t n, const integer_t m, const integer_t ku, const integer_t kl,
                                blocktype_t type, blocksection_t section);
Error_t block_Deallocate(block_t *B);
void block_SaveCSR(const char *filename, block_t *B);
block_t *block_loadCSR(const char *filename);  /* NULL on error */
/* n int32 / n values from a raw file; NULL on error; free() the result. */
integer_t *vector_LoadPermutationArray(const integer_t n, const char *filename);
complex_t *vector_LoadRHS(const integer_t n, const char *filename);

/* ---- inner-solver plugin ---- */
typedef struct {
    spike_context_t ctx;     /* own context (stream) */
    spike_factor_t factor;   /* resident factors on the device */
    integer_t n, max_nrhs;
    spike_timer_t factor_t;  /* seconds spent in directSolver_Factorize */
    spike_timer_t solve_t;   /* seconds spent in directSolver_SolveForRHS */
    integer_t rhs_block_count, rhs_column_count;
} DirectSolverHander_t;

DirectSolverHander_t *directSolver_CreateHandler(void);
/* right-hand sides per solve pass (the reference's block size) */
Error_t directSolver_Configure(DirectSolverHander_t *handler, const integer_t max_nrhs);
/* copy A to the device and factor it (mixed precision, FP64 refinement) */
Error_t directSolver_Factorize(DirectSolverHander_t *handler, const integer_t n, const integer_t nnz,
                               integer_t *colind, integer_t *rowptr, complex_t *aij);
/* x = A^{-1} b with the resident factors; x, b n x nrhs column-major (host) */
Error_t directSolver_SolveForRHS(DirectSolverHander_t *handler, const integer_t nrhs, complex_t *xij,
                                 complex_t *bij);
Error_t directSolver_ShowStatistics(DirectSolverHander_t *handler);
Error_t directSolver_Finalize(DirectSolverHander_t *handler);
/* factor + solve + release in one call */
Error_t directSolver_Solve(integer_t n, integer_t nnz, integer_t nrhs, integer_t *colind, integer_t *rowptr,
                           complex_t *aij, complex_t *xij, complex_t *bij);

#ifdef __cplusplus
}
#endif

#endif /* SPIKE_COMPAT_H */
