/*
 * spike_internal.h -- the thin C ABI between the C host layer (spike_host.c)
 * and the CUDA layer (spike_*.cu).  Plain C types only.
 *
 * Vocabulary (the reference's, OpenMP/spike_analysis.h:38-53 and
 * OpenMP/spike_interfaces.c):
 *   partition i   rows [part_start[i], part_start[i+1]) of A, m_i rows
 *   block         KB consecutive rows of a partition; KB >= max(ku, kl) is the
 *                 tile size, so A_i is block tridiagonal with KB x KB blocks
 *                 D_J (diagonal), E_J = A(J, J+1), F_J = A(J+1, J)
 *   padded rows   a partition is padded with identity rows up to N_i * KB
 *   spikes        V_i = A_i^{-1} B_i, W_i = A_i^{-1} C_i
 *   tips          top = first KB rows, bottom = last KB real rows
 *   interface i   unknowns (b_i, t_{i+1}): bottom tip of partition i and top
 *                 tip of partition i+1; the reduced system has p-1 interfaces
 */
#ifndef SPIKE_GB300_INTERNAL_H
#define SPIKE_GB300_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* value type of the caller's arrays */
enum spk_dtype { SPK_S = 0, SPK_D = 1, SPK_C = 2, SPK_Z = 3 };
/* factor precision: FP32/complex64 factors with FP64 refinement, or FP64 */
enum spk_mode { SPK_MIXED = 0, SPK_PLAIN = 1 };

/* error detail codes (spike_last_error_code) */
enum spk_err {
    SPK_OK = 0,
    SPK_EARG = 1,       /* bad argument */
    SPK_ECSR = 2,       /* invalid CSR: out-of-range or unsorted/duplicate column */
    SPK_EBAND = 3,      /* bandwidth above what the kernels support */
    SPK_ECUDA = 4,      /* a CUDA runtime call failed */
    SPK_EMEM = 5,       /* device or host allocation failed */
    SPK_EPIVOT = 6,     /* zero or non-finite pivot in a diagonal block */
    SPK_ECONV = 7,      /* refinement did not reach the tolerance */
    SPK_ENODEV = 8,     /* no CUDA device */
    SPK_EHANDLE = 9,    /* bad or released handle */
    SPK_ETIMEOUT = 10   /* a kernel gave up waiting for a bulk copy into shared memory */
};

/* kernel families timed by the phase timer */
enum spk_phase {
    SPK_PH_ANALYZE = 0,
    SPK_PH_FACTOR_FWD = 1, /* k_factor_fwd: CSR scatter + block LU + W forward sweep */
    SPK_PH_FACTOR_BWD = 2, /* k_factor_bwd + k_tips: spike backward sweeps */
    SPK_PH_RED_FACTOR = 3, /* cyclic reduction of the reduced system */
    SPK_PH_APPLY = 4,      /* k_apply + k_ytips: y = A_i^{-1} r */
    SPK_PH_RED_SOLVE = 5,  /* reduced solve with FP64 refinement */
    SPK_PH_RETRIEVE = 6,   /* k_retrieve */
    SPK_PH_RESIDUAL = 7,   /* k_residual: FP64 r = b - A x */
    SPK_PH_BAND_TILES = 8, /* k_band_tiles: CSR -> dense factor-precision tiles */
    SPK_NPHASES = 9
};
#define SPK_MAX_EVENTS 64

/* device error word bits, written by kernels with atomicOr */
#define SPK_DEV_ERR_PIVOT 1u
#define SPK_DEV_ERR_BAND 2u
#define SPK_DEV_ERR_CSR 4u
#define SPK_DEV_ERR_TIMEOUT 8u /* a bounded wait on a bulk copy gave up; the kernel returned early */

/* One system of a batch as the kernels see it.  A batch group lays its
 * systems end to end in one row space (system s owns rows [row0, row0 + n));
 * partitions never straddle two systems, so no coupling crosses a system
 * boundary and those interfaces decouple in the reduced system.  The kernels
 * read each system's own CSR, b and x through this table (no packing). */
typedef struct spk_sysref {
    const int *rowptr, *colind;
    const void *aij; /* FP64 / complex128 */
    void *x;         /* n x nrhs, ld n */
    const void *b;   /* n x nrhs, ld n */
    long long row0;  /* first row of the system in the group's row space */
    int n, pad;
} spk_sysref;

typedef struct spk_plan {
    /* problem */
    int n, nrhs_max, ku, kl, KB, p;
    int is_complex, mode;
    long long nnz;
    /* schedule (host copies) */
    int *part_start; /* p+1 */
    int *blk_off;    /* p+1, prefix sum of blocks per partition */
    int total_blocks;
    long long NP; /* padded rows = total_blocks * KB */
    int n_iface;  /* p - 1 */
    /* two-sided partition solves (spike_twist.cu): every partition is
     * eliminated from both ends towards its block M = N_i / 2 */
    int twist, twist_cap; /* in use / possible for this schedule and precision */
    /* the reduced system's cyclic reduction in FP64 (complex128) even when
     * the partitions' factors are FP32 (SPIKE_OPT_REDUCED_FP64; tiles up to
     * 64 rows).  The cyclic-reduction arrays are allocated with 8-byte
     * (16-byte complex) scalars whatever the mode, so a call may switch. */
    int red_fp64;
    /* k_band_tiles also validates the CSR and measures the bandwidth into
     * d_err[1..2] (set when the separate analysis pass was skipped) */
    int validate;
    /* impl_cols: the device holds no column indices for this call -- the host
     * verified that every row r is the full band, columns max(0, r - impl_kl)
     * .. min(n - 1, r + ku) -- so the band tiles and the residual derive the
     * column of entry t of row r as max(0, r - impl_kl) + (t - rowptr[r]) */
    int impl_cols, impl_kl;
    /* the first right-hand-side chunk's y = A_i^{-1} b already ran (next to
     * the reduced factorization, on another stream) */
    int first_applied;
    /* device copies of the schedule */
    int *d_part_start, *d_blk_off;
    int *d_blk_part; /* total_blocks: partition of each block */
    /* factor-precision arrays, [total_blocks][KB][KB] (row-major tiles) */
    void *d_L, *d_G, *d_E, *d_V, *d_W; /* V, W tiles are column-major */
    void *d_Bhat;                      /* [p][KB][KB] */
    void *d_T;                         /* [total_blocks][3][KB][KB]: D, F^T, E per block (row-major) */
    /* reduced system: level-0 quadrant blocks in FP64 (or complex128) */
    void *d_RP, *d_RQ, *d_RX, *d_RY; /* [n_iface][KB][KB] */
    /* cyclic reduction factors in factor precision */
    int cr_levels;
    int *cr_count;    /* blocks at each level (host), cr_levels+1 entries */
    long long *cr_off; /* offset (in tiles) of each level's block arrays */
    long long *cr_moff; /* offset (in tiles) of each level's odd-block M arrays */
    void *d_crP, *d_crQ, *d_crX, *d_crY; /* all levels, factor precision */
    void *d_crM;                         /* 4 tiles per odd block: M00 M01 M10 M11 */
    void *d_crg;                         /* per-level reduced RHS work, factor precision */
    long long crg_stride;                /* elements per RHS column of d_crg */
    /* right-hand-side work (per solve) */
    void *d_z, *d_y;       /* factor precision, NP x nrhs_max */
    void *d_g, *d_u, *d_rr; /* FP64 reduced RHS, solution, reduced residual: n_iface*2KB x nrhs_max */
    void *d_du;            /* FP64 reduced correction */
    unsigned int *d_err;   /* device error word */
    /* batch groups only (NULL otherwise): per-system table and the system
     * of each partition; CSR, b and x are then read through the table */
    const spk_sysref *d_sys;
    const int *d_part_sys;
    double *d_norms;       /* 2*nrhs_max: ||r||^2 then ||b||^2 per column */
    /* bookkeeping */
    void *astream;      /* allocations stream-ordered on this stream (NULL: cudaMalloc) */
    long long launches; /* kernel launches issued for this plan */
    size_t bytes;       /* device bytes held */
    /* optional per-phase CUDA-event timing (SPIKE_OPT_PHASE_TIMING) */
    int timing;
    void *ev;                          /* SPK_MAX_EVENTS cudaEvent_t pairs */
    int ev_phase[SPK_MAX_EVENTS];
    int nev;
    double phase_ms[SPK_NPHASES];
    long long phase_calls[SPK_NPHASES];
} spk_plan;

/* phase timing: begin/end record events on the stream; collect (after a
 * stream synchronize) adds the elapsed times to phase_ms / phase_calls */
void spk_phase_begin(spk_plan *P, int phase, void *stream);
void spk_phase_end(spk_plan *P, void *stream);
int spk_phase_collect(spk_plan *P);
void spk_phase_destroy(spk_plan *P);

/* ---- fixed workspace of the no-allocation solve (spike_noalloc.cu) ---- */
#define SPK_NOALLOC_SCRATCH_BYTES (32u << 20) /* 32 MiB per device */
/* device address of the fixed workspace on the current device, resolved with
 * cudaGetSymbolAddress on every call */
int spk_noalloc_scratch(void **ptr, size_t *bytes);

/* ---- device / memory (spike_util.cu) ---- */
int spk_device_count(void);
int spk_current_device(void);
int spk_sm_count(void);
int spk_set_device(int dev);
int spk_mem_info(size_t *free_b, size_t *total_b);
int spk_malloc(void **p, size_t bytes);
void spk_free(void *p);
/* stream-ordered when stream != NULL (cudaMallocAsync / cudaFreeAsync) */
int spk_malloc_on(void **p, size_t bytes, void *stream);
void spk_free_on(void *p, void *stream);
int spk_host_register(void *p, size_t bytes);
int spk_host_unregister(void *p);
int spk_stream_create(void **stream);
void spk_stream_destroy(void *stream);
int spk_stream_sync(void *stream);
int spk_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream);
int spk_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream);
int spk_memcpy_d2d(void *dst, const void *src, size_t bytes, void *stream);
/* height rows of width bytes, dpitch / spitch apart, host or device either side */
int spk_memcpy_2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height, void *stream);
/* page-locked host memory */
int spk_host_alloc(void **p, size_t bytes);
void spk_host_free(void *p);
int spk_memset(void *dst, int v, size_t bytes, void *stream);
const char *spk_cuda_error_string(void);

/* ---- analysis, conversion, residual (spike_util.cu) ---- */
/* bandwidth and CSR validation on the device; out[0] = ku, out[1] = kl,
 * out[2] = error flags (SPK_DEV_ERR_CSR).  d_scratch: 4 device ints.
 * Synchronizes the stream. */
int spk_analyze(int n, long long nnz, const int *d_rowptr, const int *d_colind, int *d_scratch, int *out,
                void *stream, long long *launches);
/* sharded solve: bandwidth of rows [row0, row0 + m) held with global columns
 * into d_out (4 device ints: [0] = ku, [1] = kl, [2] = 1 on a bad row pointer
 * or column), queued on the stream; and the rank's local CSR, in place, with
 * h identity rows either side (k_shard_local) */
int spk_rows_band(int m, long long nnz, int row0, int n, const int *d_rowptr, const int *d_colind, int *d_out,
                  void *stream);
int spk_shard_local(int m, long long nnz, int h, int row0, int *d_rowptr, int *d_colind, double *d_aij, void *stream);
/* widen caller values to FP64 / complex128 (S -> D, C -> Z) and narrow back */
int spk_widen(const void *src, void *dst, long long count, int is_complex, void *stream, long long *launches);
int spk_narrow(const void *src, void *dst, long long count, int is_complex, void *stream, long long *launches);
/* r = b - A x for every column (FP64 / complex128), ||r||^2 per column into
 * norms[0:nrhs]; when want_bnorm, ||b||^2 into norms[nrhs:2*nrhs]. */
int spk_residual(const spk_plan *P, const int *d_rowptr, const int *d_colind, const void *d_aij,
                 const void *d_x, const void *d_b, void *d_r, int nrhs, int want_bnorm, double *d_norms,
                 void *stream);

/* Batch residual in FP64 / complex128 over the systems of a group, one CTA
 * per chunk of rows of one system (d_chunks: {system, first local row} pairs,
 * rows_per_chunk rows each).  have_x = 0: r = b (x is zero); 1: r = b - A x.
 * r: the group's row space, ld n_rows.  norms[s][0:nrhs] += ||r||^2 and
 * norms[s][nrhs:2 nrhs] += ||b||^2. */
int spk_residual_batch(const spk_sysref *d_sys, const int *d_chunks, int nchunks, int rows_per_chunk,
                       int row_len, long long n_rows, int nrhs, int is_complex, int have_x, void *d_r,
                       double *d_norms, void *stream, long long *launches);
/* relres[s] = max_h ||r_h|| / ||b_h|| from the norms above; *d_worst =
 * max over s (as double bits, atomically) */
int spk_batch_relres(const double *d_norms, int nsys, int nrhs, double *d_relres, unsigned long long *d_worst,
                     void *stream, long long *launches);

/* ---- CUDA graphs and stream fork/join (spike_util.cu) ---- */
int spk_capture_begin(void *stream);
int spk_capture_end(void *stream, void **graph_exec);
int spk_graph_launch(void *graph_exec, void *stream);
void spk_graph_destroy(void *graph_exec);
/* make `child` wait for the work issued so far on `parent` */
int spk_stream_fork(void *parent, void *child);
/* events without timing: record on a stream, make another stream wait */
int spk_event_create(void **event);
void spk_event_destroy(void *event);
int spk_event_record(void *event, void *stream);
int spk_stream_wait_event(void *stream, void *event);
/* timing with an event pair on one stream (ms between begin and end) */
int spk_timer_begin(void **timer, void *stream);
int spk_timer_end(void *timer, void *stream, double *ms);

/* ---- factorization (spike_factor.cu) ---- */
/* K2: block LU of every A_i, spikes V_i/W_i, tips into the reduced blocks. */
int spk_factor(spk_plan *P, const int *d_rowptr, const int *d_colind, const void *d_aij, void *stream);
/* shared-memory bytes the factor kernels need for this plan (0 = unsupported) */
size_t spk_factor_smem(int KB, int is_complex, int mode);

/* ---- two-sided partition factorization (spike_twist.cu) ---- */
/* 1 if the two-sided kernels exist for this tile size and precision */
int spk_twist_supported(int KB, int is_complex, int mode);
/* Partitions [part0, part1): forward = 1: both elimination chains, the
 * spikes' forward sweeps and the middle block; forward = 0: the spikes' back
 * substitution */
int spk_twist_factor(spk_plan *P, int forward, int part0, int part1, void *stream);
/* The factorization of a two-sided plan in pieces, for copies that arrive in
 * partition ranges: band tiles, chains and back substitution of partitions
 * [part0, part1) (their CSR rows must be on the device), then, after the
 * last range, the tips. */
int spk_factor_range(spk_plan *P, const int *d_rowptr, const int *d_colind, const void *d_aij, int part0, int part1,
                     void *stream);
int spk_factor_tips(spk_plan *P, void *stream);

/* ---- reduced system (spike_reduced.cu) ---- */
int spk_reduced_factor(spk_plan *P, void *stream);
/* u = R^{-1} g for nrhs columns (FP64), with refine_iters FP64 refinement
 * sweeps around the factor-precision cyclic reduction. */
int spk_reduced_solve(spk_plan *P, int nrhs, int refine_iters, void *stream);

/* ---- right-hand-side sweeps (spike_apply.cu) ---- */
/* y_i = A_i^{-1} r_i for every partition (r in FP64 / complex128, caller
 * layout n x nrhs, ld n), y tips into the reduced RHS d_g. */
int spk_apply(spk_plan *P, const void *d_r, int nrhs, void *stream);
/* x += y - V_i t_{i+1} - W_i b_{i-1} (x in FP64 / complex128, ld n). */
int spk_retrieve(spk_plan *P, void *d_x, int nrhs, int accumulate, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SPIKE_GB300_INTERNAL_H */
