/*
 * spike_interfaces.h -- the drop-in C API of the SPIKE banded solver.
 *
 * Same five entry points, argument order and meaning as the reference's
 * OpenMP/spike_interfaces.h:28-72:
 *
 *   A is a square n x n matrix in 0-based CSR (rowptr[n+1], colind[nnz],
 *   aij[nnz]); columns inside a row must be strictly increasing.  Its
 *   bandwidth (ku, kl) is read from the pattern, as the reference does in
 *   OpenMP/spike_matrix.c:258.  b (bij) and x (xij) are dense column-major
 *   n x nrhs arrays with leading dimension n.  b is not modified; x is fully
 *   overwritten.  The caller owns all five arrays.
 *
 * Differences from the reference, all intentional:
 *   - sspike/cspike/zspike solve (the reference's are stubs that return
 *     success without touching x: OpenMP/spike_interfaces.c:3-39);
 *   - every error returns SPIKE_ERROR instead of calling abort()
 *     (OpenMP/spike_interfaces.c:53-56); spike_last_error() in
 *     spike_gb300.h gives the detail;
 *   - every right-hand side column is written (the reference copies column 0
 *     of each partition into all columns: OpenMP/spike_matrix.c:1341-1342).
 *
 * The solve runs on the current CUDA device (hand-written sm_103a kernels);
 * there is no CPU fallback.  The calls are blocking and thread-safe (each
 * host thread gets its own default context and CUDA stream).
 */
#ifndef SPIKE_GB300_INTERFACES_H
#define SPIKE_GB300_INTERFACES_H

#include "spike_datatypes.h"

#ifdef __cplusplus
extern "C" {
#endif

/* OpenMP/spike_interfaces.h:24-25 */
typedef struct { float  real; float  imag; } complex8;
typedef struct { double real; double imag; } complex16;

/* Replaces OpenMP/spike_interfaces.h:28-35 (a stub in the reference). */
Error_t sspike_core_host(const integer_t n, const integer_t nnz, const integer_t nrhs,
                         integer_t *colind, integer_t *rowptr,
                         float *aij, float *xij, float *bij);

/* Replaces OpenMP/spike_interfaces.h:37-44 (OpenMP/spike_interfaces.c:43-419). */
Error_t dspike_core_host(const integer_t n, const integer_t nnz, const integer_t nrhs,
                         integer_t *colind, integer_t *rowptr,
                         double *aij, double *xij, double *bij);

/* Replaces OpenMP/spike_interfaces.h:46-53 (a stub in the reference). */
Error_t cspike_core_host(const integer_t n, const integer_t nnz, const integer_t nrhs,
                         integer_t *colind, integer_t *rowptr,
                         complex8 *aij, complex8 *xij, complex8 *bij);

/* Replaces OpenMP/spike_interfaces.h:55-62 (a stub in the reference). */
Error_t zspike_core_host(const integer_t n, const integer_t nnz, const integer_t nrhs,
                         integer_t *colind, integer_t *rowptr,
                         complex16 *aij, complex16 *xij, complex16 *bij);

/* Replaces OpenMP/spike_interfaces.h:64-71 (OpenMP/spike_interfaces.c:421-1091).
 * The reference processes right-hand sides in chunks of 200 columns to bound
 * host memory; on the device the chunking is internal, so this entry point
 * returns exactly what dspike_core_host returns. */
Error_t dspike_core_host_blocking(const integer_t n, const integer_t nnz, const integer_t nrhs,
                                  integer_t *colind, integer_t *rowptr,
                                  double *aij, double *xij, double *bij);

#ifdef __cplusplus
}
#endif

#endif /* SPIKE_GB300_INTERFACES_H */
