/*
 * spike_gb300.h -- additive extensions to the SPIKE C API.
 *
 * Nothing here changes spike_interfaces.h; a caller written against the
 * reference's API needs none of it.  The extensions expose what the
 * reference keeps internal or compile-time:
 *
 *   - options (precision mode, partition count, refinement) that the
 *     reference fixes in code: p = 4 (OpenMP/spike_analysis.c:168), the
 *     -D_DATATYPE_ scalar type (OpenMP/spike_datatypes.h:29-84);
 *   - error detail: the reference aborts (OpenMP/spike_interfaces.c:53-56),
 *     this library returns SPIKE_ERROR and records why;
 *   - factor handles: factor once, solve many right-hand sides with the
 *     factors resident on the device (the reference re-factors every block
 *     in the retrieval phase, OpenMP/spike_interfaces.c:271-277);
 *   - device-pointer entry points for callers whose data already sits in HBM;
 *   - contexts bound to a caller-chosen CUDA stream.
 *
 * A NULL context everywhere means the calling host thread's default context
 * (the one the spike_interfaces.h entry points use).
 */
#ifndef SPIKE_GB300_H
#define SPIKE_GB300_H

#include "spike_interfaces.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct spike_context_s *spike_context_t;
typedef struct spike_factor_s *spike_factor_t;

/* ---- options (spike_set_option) ---- */
#define SPIKE_OPT_PRECISION 0      /* SPIKE_PRECISION_MIXED (default) or _FP64 */
#define SPIKE_OPT_PARTITIONS 1     /* 0 = automatic (default), else p */
#define SPIKE_OPT_MAX_REFINE 2     /* correction sweeps after the first solve (default 3) */
#define SPIKE_OPT_TOLERANCE 3      /* relative residual target (default 1e-12) */
#define SPIKE_OPT_REDUCED_REFINE 4 /* FP64 refinement sweeps on the reduced system (default 2 mixed, 1 FP64) */
#define SPIKE_OPT_PHASE_TIMING 5   /* 1 = time each kernel family with CUDA events (default 0) */
#define SPIKE_OPT_STREAM_ALLOC 6   /* 1 = workspace via cudaMallocAsync on the context's stream, so contexts on
                                      different streams overlap while they allocate (default 0) */
#define SPIKE_OPT_TWIST 7          /* 1 = eliminate each partition from both ends at once where the kernels
                                      allow it (tiles 16..64 fitting four CTAs per SM, >= 8 blocks per
                                      partition); 0 = top-down only (default 1) */
#define SPIKE_OPT_REDUCED_FP64 9   /* 1 = the reduced system's cyclic reduction in FP64 (complex128) also in
                                      mixed precision, for tiles up to 64 rows (the reference solves R in FP64
                                      with PARDISO, OpenMP/spike_algebra.c:263-420); 0 = in the factors'
                                      precision, FP64 refinement sweeps on R making up the rest (default 0) */
#define SPIKE_OPT_HOST_THREADS 8   /* host threads that, in a call with host arrays whose plan is reused,
                                      check that the CSR is the full band while its values travel, so
                                      the column indices stay on the host (default 8; 0 = always copy
                                      them) */

#define SPIKE_PRECISION_MIXED 0 /* FP32 / complex64 factors, FP64 residual + update + reduced solve */
#define SPIKE_PRECISION_FP64 1  /* FP64 / complex128 everywhere */

/* ---- error detail ---- */
#define SPIKE_ERR_NONE 0
#define SPIKE_ERR_ARGUMENT 1
#define SPIKE_ERR_CSR 2        /* out-of-range, unsorted or duplicate column index, bad rowptr */
#define SPIKE_ERR_BANDWIDTH 3  /* max(ku, kl) above the supported tile size */
#define SPIKE_ERR_CUDA 4
#define SPIKE_ERR_MEMORY 5
#define SPIKE_ERR_PIVOT 6      /* zero or non-finite pivot: A is not diagonally dominant enough */
#define SPIKE_ERR_CONVERGENCE 7 /* refinement stopped above the tolerance (x holds the last iterate) */
#define SPIKE_ERR_NO_DEVICE 8
#define SPIKE_ERR_HANDLE 9
#define SPIKE_ERR_BUSY 10       /* a server's admission queue was full (spike_server_config_t.max_queue) */

int spike_last_error_code(void);          /* of the calling thread's last call */
const char *spike_last_error(void);       /* human-readable, thread-local */

/* ---- contexts ---- */
Error_t spike_context_create(spike_context_t *ctx);          /* on the current CUDA device */
/* Factor handles and batches created on a context keep it alive: destroying
 * the context before releasing them drops the caller's reference only, and
 * the context goes with the last of them. */
Error_t spike_context_destroy(spike_context_t ctx);
/* Run this context's work on a caller-owned cudaStream_t (NULL = own stream). */
Error_t spike_context_set_stream(spike_context_t ctx, void *cuda_stream);
Error_t spike_set_option(spike_context_t ctx, int option, double value);
Error_t spike_get_option(spike_context_t ctx, int option, double *value);

/* Statistics of the context's last solve. */
typedef struct {
    double relres_max;        /* max over columns of ||b - A x|| / ||b|| (FP64) */
    int refine_sweeps;        /* correction sweeps after the first solve */
    int partitions, ku, kl, block;
    long long kernel_launches; /* kernels launched by the last call */
    size_t device_bytes;      /* device memory held by the context's plan */
    int twisted;              /* 1 if the partitions were eliminated from both ends (SPIKE_OPT_TWIST) */
    int columns_implied;      /* 1 if the column indices stayed on the host (full band, SPIKE_OPT_HOST_THREADS) */
    int reduced_fp64;         /* 1 if the reduced system was factored and solved in FP64 (SPIKE_OPT_REDUCED_FP64) */
} spike_info_t;
Error_t spike_get_info(spike_context_t ctx, spike_info_t *info);

/* Per-kernel-family device time accumulated while SPIKE_OPT_PHASE_TIMING is
 * on, measured with CUDA events on the context's stream.  Families, in order:
 *   0 analysis, 1 factor forward (block LU + W sweep),
 *   2 factor backward (spike sweeps + tips), 3 reduced factorization,
 *   4 right-hand-side sweeps, 5 reduced solve, 6 retrieval, 7 FP64 residual,
 *   8 band tiles (CSR -> dense tiles).
 * ms[i] is the summed time and calls[i] the number of timed launches of
 * family i (nphases <= 9); reset = 1 clears the accumulators afterwards. */
#define SPIKE_NUM_PHASES 9
Error_t spike_get_phase_times(spike_context_t ctx, int nphases, double *ms, long long *calls, int reset);

/* ---- host-array solves on an explicit context ---- */
/* dspike_core_host / zspike_core_host on an explicit context (host arrays,
 * same meaning; NULL = the calling thread's default context). */
Error_t spike_dsolve(spike_context_t ctx, integer_t n, integer_t nnz, integer_t nrhs, const integer_t *colind,
                     const integer_t *rowptr, const double *aij, double *x, const double *b);
Error_t spike_zsolve(spike_context_t ctx, integer_t n, integer_t nnz, integer_t nrhs, const integer_t *colind,
                     const integer_t *rowptr, const void *aij, void *x, const void *b);

/* ---- device-pointer solves: every array already in device memory ---- */
Error_t spike_dsolve_device(spike_context_t ctx, integer_t n, integer_t nnz, integer_t nrhs,
                            const integer_t *d_colind, const integer_t *d_rowptr, const double *d_aij,
                            double *d_x, const double *d_b);
Error_t spike_zsolve_device(spike_context_t ctx, integer_t n, integer_t nnz, integer_t nrhs,
                            const integer_t *d_colind, const integer_t *d_rowptr, const complex16 *d_aij,
                            complex16 *d_x, const complex16 *d_b);

/* ---- solve without device allocation ----
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they solve: programs whose own pool allocator has taken the
 * device heap (a library's cudaMalloc would fail or fragment it), latency-
 * critical loops that cannot absorb the device-wide synchronisation of
 * cudaFree, and plugin hosts that do not let a library allocate on their
 * behalf.  Same meaning as spike_dsolve_device (device arrays, mixed precision,
 * FP64 refinement to 1e-12, automatic partitions), but every temporary lives in
 * one fixed workspace of SPIKE_NOALLOC_WORKSPACE_BYTES that the library keeps
 * on each device that loads it, for the life of the process; no context is
 * used and nothing is allocated, on the device or the host.  Work runs on
 * `cuda_stream` (NULL = the legacy default stream); the call synchronises that
 * stream (after the bandwidth analysis and after each residual) and returns
 * when the solve is done.
 *   - A system whose workspace exceeds the fixed size (roughly n * max(ku,kl)
 *     past a few million, e.g. n = 100,000 with ku = kl = 8) is rejected with
 *     SPIKE_ERR_MEMORY once the bandwidth analysis -- the only work queued
 *     before the check -- has fixed its tile size.
 *   - All calls on a device share the workspace and it keeps the previous
 *     call's contents (the solve clears what it needs cleared).  Calls whose
 *     GPU work overlaps -- from two host threads, or on two streams -- race on
 *     it: serialise them. */
#define SPIKE_NOALLOC_WORKSPACE_BYTES (32u << 20)
Error_t spike_dsolve_device_noalloc(integer_t n, integer_t nnz, integer_t nrhs, const integer_t *d_colind,
                                    const integer_t *d_rowptr, const double *d_aij, double *d_x, const double *d_b,
                                    void *cuda_stream);

/* ---- factor handles ---- */
/* Host arrays: the handle copies A to the device and owns the copy. */
Error_t spike_dfactor(spike_context_t ctx, integer_t n, integer_t nnz, const integer_t *colind,
                      const integer_t *rowptr, const double *aij, spike_factor_t *f);
Error_t spike_zfactor(spike_context_t ctx, integer_t n, integer_t nnz, const integer_t *colind,
                      const integer_t *rowptr, const complex16 *aij, spike_factor_t *f);
/* Device arrays: the handle references them; keep them alive until release. */
Error_t spike_dfactor_device(spike_context_t ctx, integer_t n, integer_t nnz, const integer_t *d_colind,
                             const integer_t *d_rowptr, const double *d_aij, spike_factor_t *f);
/* Solve with resident factors; x, b host (column-major, ld n). */
Error_t spike_dsolve_factored(spike_factor_t f, integer_t nrhs, double *x, const double *b);
Error_t spike_zsolve_factored(spike_factor_t f, integer_t nrhs, complex16 *x, const complex16 *b);
/* Same with device arrays. */
Error_t spike_dsolve_factored_device(spike_factor_t f, integer_t nrhs, double *d_x, const double *d_b);
Error_t spike_factor_release(spike_factor_t f);

/* ---- batches of independent systems ----
 * No counterpart in the reference (one system per dspike_core_host call).
 * Thousands of systems of uneven n, bandwidth and nrhs are solved by one CUDA
 * graph launch: the systems are grouped by tile size and nrhs, each group is
 * one SPIKE schedule whose partitions never straddle two systems, and every
 * group runs on its own stream inside the graph.  Mixed or FP64 precision,
 * tolerance and refinement limit come from the context. */
typedef struct spike_batch_s *spike_batch_t;
typedef struct {
    integer_t n, nnz, nrhs;           /* nrhs in [1, 32] */
    const integer_t *d_colind, *d_rowptr; /* device, CSR 0-based, sorted rows */
    const double *d_aij;                  /* device */
    double *d_x;                          /* device, n x nrhs column-major (output) */
    const double *d_b;                    /* device, n x nrhs column-major */
} spike_dsystem_t;

#define SPIKE_BATCH_AUTOTUNE 1 /* time candidate tile sizes and partition lengths per group */
#define SPIKE_BATCH_NO_GRAPH 2 /* launch eagerly on every run instead of replaying the graph */

/* Plan a batch: read every pattern (bandwidth, CSR validity), group, choose
 * the schedules (autotuned with SPIKE_BATCH_AUTOTUNE, else by rule), allocate,
 * run once (the warm-up fixes how many refinement sweeps the graph holds) and
 * capture the solve as one graph.  The descriptors are copied; the arrays are
 * read at every run, so A's values and b may change between runs, the pattern
 * and the pointers may not. */
Error_t spike_dbatch_create(spike_context_t ctx, integer_t count, const spike_dsystem_t *systems, int flags,
                            spike_batch_t *out);
/* Solve every system: one graph launch after the work already queued on the
 * context's stream; a group still above the tolerance then gets eager
 * refinement sweeps up to the context's limit.  Returns after the solve. */
Error_t spike_batch_run(spike_batch_t batch);
/* Relative residual max_h ||b_h - A x_h|| / ||b_h|| of every system after the
 * last run (count entries, in the systems' order). */
Error_t spike_batch_relres(spike_batch_t batch, double *relres);
typedef struct {
    int systems, groups;
    int graph;                        /* 1 when runs replay a captured graph */
    int graph_sweeps;                 /* most refinement sweeps any group's graph holds */
    int extra_sweeps;                 /* eager sweeps the last run added */
    double relres_max;                /* worst relative residual of the last run */
    long long graph_kernel_launches;  /* kernels in one graph launch */
    size_t device_bytes;
    double tune_ms;                   /* device time spent timing candidates */
} spike_batch_info_t;
Error_t spike_batch_get_info(spike_batch_t batch, spike_batch_info_t *info);
typedef struct {
    int block, nrhs, bandwidth, systems, partitions, rows_per_partition, graph_sweeps;
    long long rows, nnz;
} spike_batch_group_t;
Error_t spike_batch_group(spike_batch_t batch, integer_t i, spike_batch_group_t *group);
Error_t spike_batch_destroy(spike_batch_t batch);
/* The partition rule of a batch (host only): partitions of a system of n
 * rows with tile size KB at a target of rows_per_partition rows -- the
 * nearest count, at least 1 and at most n / (2 KB); the partitions then
 * start at multiples of floor(n / p), the remainder going to the last. */
integer_t spike_batch_partitions(integer_t n, integer_t KB, integer_t rows_per_partition);

/* ---- serving: a request loop with continuous batching ----
 * No counterpart in the reference.  `slots` worker threads, each with its own
 * context and stream (workspace stream-ordered), take requests from a FIFO as
 * soon as a slot is free and the request's device footprint fits in the
 * budget left by running requests; their GPU work overlaps.  Requests with a
 * factor key keep their factorization resident (LRU cache with its own budget)
 * and later requests with the same key solve with it.  Host arrays; they must
 * stay valid until the request is done. */
typedef struct spike_server_s *spike_server_t;
typedef struct {
    int slots;           /* concurrent requests (1..64) */
    int precision;       /* SPIKE_PRECISION_MIXED or _FP64 */
    double tolerance;    /* relative residual target (0 = 1e-12) */
    int max_refine;      /* refinement sweeps (0 = 3) */
    size_t hbm_budget;   /* device bytes for running requests (0 = 60 % of free memory) */
    size_t cache_budget; /* device bytes for resident factors (0 = 20 % of free memory) */
    int max_queue;       /* requests waiting for a slot beyond which a new request is completed at once with
                            SPIKE_ERR_BUSY (load shedding; 0 = an unbounded queue) */
} spike_server_config_t;
typedef struct {
    integer_t n, nnz, nrhs;
    const integer_t *colind, *rowptr;
    const double *aij;
    const double *b; /* n x nrhs column-major */
    double *x;       /* n x nrhs column-major (output) */
    integer_t bandwidth; /* max(ku, kl) when known, else -1 (scanned from the pattern) */
    long long factor_key; /* >= 0: keep / reuse the factorization under this key; -1: none */
    double arrival;      /* arrival time on spike_server_clock, < 0 = at submission */
} spike_request_t;
typedef struct {
    int done, error_code;
    double relres;
    int sweeps, factor_hit;
    double t_arrival, t_admit, t_done; /* spike_server_clock seconds */
    size_t footprint;                  /* device bytes charged while it ran */
} spike_request_status_t;
typedef struct {
    long long submitted, completed, rejected, failed, queued;
    long long factor_hits, factor_misses;
    int running, peak_running, resident_factors;
    size_t device_bytes_running, device_bytes_cached;
    double latency_p50, latency_p99, latency_max; /* seconds, arrival to completion */
    double mean_queue_wait, throughput;           /* seconds; completed per second */
    double relres_max;
    long long rejected_busy; /* of `rejected`: turned away because the queue was full */
} spike_server_stats_t;
Error_t spike_server_create(const spike_server_config_t *cfg, spike_server_t *server);
/* Queue a request; a request larger than the whole budget (or with a band
 * above the largest tile) is completed at once with an error. */
Error_t spike_server_submit(spike_server_t server, const spike_request_t *req, long long *ticket);
/* Block until the request is done; returns its error, if any. */
Error_t spike_server_wait(spike_server_t server, long long ticket, spike_request_status_t *status);
/* The request's status now, without waiting (status->done = 0 while it is queued or running). */
Error_t spike_server_poll(spike_server_t server, long long ticket, spike_request_status_t *status);
Error_t spike_server_drain(spike_server_t server);
Error_t spike_server_stats(spike_server_t server, spike_server_stats_t *stats);
double spike_server_clock(spike_server_t server); /* seconds since creation */
Error_t spike_server_destroy(spike_server_t server); /* drains first */

/* ---- bandwidth-reducing reordering (host) ----
 * The reference reorders with cuSolverSp's host RCM + csrperm
 * (cuda_standalone_symrcm, OpenMP/spike_cuda.c:898-971) and permutes vectors
 * with permute_vector (OpenMP/spike_algebra.c:34-53). */
/* Reverse Cuthill-McKee order of the pattern of A + A^T: new row i is old row
 * perm[i]. */
Error_t spike_rcm_permutation(integer_t n, integer_t nnz, const integer_t *colind, const integer_t *rowptr,
                              integer_t *perm);
/* B = A(perm, perm) into caller arrays (same nnz), rows sorted by column. */
Error_t spike_permute_csr(integer_t n, integer_t nnz, const integer_t *colind, const integer_t *rowptr,
                          const double *aij, const integer_t *perm, integer_t *out_colind, integer_t *out_rowptr,
                          double *out_aij);
/* permute_vector's meaning for nrhs columns: flag > 0 -> v = v(perm),
 * flag <= 0 -> v(perm) = v. */
Error_t spike_permute_vector(integer_t flag, integer_t n, integer_t nrhs, const integer_t *perm, double *v);
/* Solve A x = b for a general sparse A: RCM, permute, banded solve on the
 * device, permute back.  perm_out (optional, n entries) receives the order. */
Error_t spike_dsolve_reordered(spike_context_t ctx, integer_t n, integer_t nnz, integer_t nrhs,
                               const integer_t *colind, const integer_t *rowptr, const double *aij, double *x,
                               const double *b, integer_t *perm_out);

/* ---- one system's partitions sharded across ranks (processes, one GPU each) ----
 * Replaces the reference's distributed SPIKE (MPI/spike_dm.c:21-202: the
 * master scatters A_i, f_i, B_i, C_i to workers, gathers their tips, solves
 * the reduced system and scatters the x tips back, MPI/spike_mpi.c:450-674).
 * Here rank r holds the CSR rows of a contiguous range of the p partitions
 * (spike_shard_range) and factors them on its own GPU, couplings to the
 * neighbouring ranks' rows included; the only exchanges are the tips of the
 * reduced system (gathered to rank 0, which solves it, and its solution
 * scattered back), one band of x rows with each neighbour before every FP64
 * residual, and the residual norms.  The transport is the caller's: the
 * library calls these functions on host buffers, in the same order on every
 * rank (NCCL, MPI, a torch.distributed group ...).  Each returns 0 on success. */
typedef struct {
    int rank, size; /* this rank and the number of ranks */
    void *user;     /* handed back to every callback */
    /* rank r's `bytes` bytes into `recv` on rank 0 at offset r * bytes (recv unused on other ranks) */
    int (*gather)(void *user, const void *send, size_t bytes, void *recv);
    /* rank 0's `send` bytes [r * bytes, (r + 1) * bytes) into rank r's `recv` (send unused on other ranks) */
    int (*scatter)(void *user, const void *send, size_t bytes, void *recv);
    /* element-wise sum of `count` doubles over all ranks, in place, the result on every rank */
    int (*allreduce_sum)(void *user, double *buf, int count);
    /* `bytes` bytes each way with both neighbours: to_lo -> rank - 1 (its from_hi), to_hi -> rank + 1 (its
     * from_lo); a neighbour that does not exist sends and receives nothing */
    int (*exchange)(void *user, const void *to_lo, const void *to_hi, void *from_lo, void *from_hi, size_t bytes);
} spike_comm_t;

/* The rows and partitions rank `rank` of `size` holds: partitions
 * [*part0, *part1) = [p rank / size, p (rank + 1) / size) and their rows
 * [*row0, *row1), partition i starting at row i floor(n / p) (the reference's
 * rule, OpenMP/spike_analysis.c:38-76; the last one takes the remainder). */
Error_t spike_shard_range(integer_t n, integer_t p, integer_t size, integer_t rank, integer_t *part0, integer_t *part1,
                          integer_t *row0, integer_t *row1);
/* Collective solve of A x = b over all ranks of `comm`: every rank passes
 * its rows [row0, row1) of A -- rowptr (rows + 1 entries, starting at 0),
 * colind (GLOBAL column indices), aij -- and of b (rows x nrhs, column-major,
 * ld = rows), and receives the same rows of x.  Mixed precision or FP64 and
 * the tolerance come from the context (the partition count is `p`, every
 * partition at least two tiles long); nrhs <= 64 per call.  Returns the same
 * status on every rank (an error on one rank is reported on all).  The
 * context keeps this rank's plans, device copy of its rows and page-locked
 * staging for the next call of the same shape (n, p, nrhs, rows, nnz, ranks);
 * a call of another shape, a failed call or spike_context_destroy frees them. */
Error_t spike_shard_dsolve(spike_context_t ctx, const spike_comm_t *comm, integer_t n, integer_t p, integer_t nrhs,
                           integer_t rows, integer_t nnz, const integer_t *colind, const integer_t *rowptr,
                           const double *aij, double *x, const double *b);
/* The routing of the reduced system's records between ranks (host only, also
 * used inside spike_shard_dsolve).  A record belongs to one interface
 * (between partitions i and i + 1) and holds left_len values that partition i
 * produces (its bottom tips) followed by right_len values that partition
 * i + 1 produces (its top tips).  Rank r's slot holds ceil(p / size) + 1
 * records: those of its local interfaces j = 0 .. part1 - part0, interface j
 * being the global interface part0 - 1 + j (j = 0 and j = part1 - part0 are
 * the interfaces with the neighbouring ranks, of which this rank knows one
 * side only).
 *   assemble: the p - 1 global records from all ranks' slots (rank 0, after
 *             a gather), each half from the rank that owns its partition;
 *   split:    every rank's slot from the global records (rank 0, before a
 *             scatter), whole records, zeros where no global interface exists. */
Error_t spike_shard_assemble(integer_t p, integer_t size, integer_t left_len, integer_t right_len,
                             const double *slots, double *global);
Error_t spike_shard_split(integer_t p, integer_t size, integer_t left_len, integer_t right_len, const double *global,
                          double *slots);

/* ---- host check of the full-band layout ----
 * *full = 1 when row r of the CSR holds exactly the columns
 * max(0, r - kl) .. min(n - 1, r + ku) in increasing order, for every row
 * (rowptr[0] = 0, rowptr[n] = nnz) -- the layout for which a solve with host
 * arrays leaves the column indices on the host (spike_info_t.columns_implied)
 * -- else 0.  Reads only rowptr[0..n] and the colind entries they delimit. */
Error_t spike_csr_full_band(integer_t n, integer_t nnz, integer_t ku, integer_t kl, const integer_t *colind,
                            const integer_t *rowptr, int *full);

#ifdef __cplusplus
}
#endif

#endif /* SPIKE_GB300_H */
