/*
 * spike_host_internal.h -- pieces of the C host layer shared by its
 * translation units (spike_host.c: the single-system API; spike_batch.c:
 * batches; spike_serve.c: the request loop).  Everything here is hidden from
 * the shared library's export table.
 */
#ifndef SPIKE_GB300_HOST_INTERNAL_H
#define SPIKE_GB300_HOST_INTERNAL_H

#include "spike_gb300.h"
#include "spike_internal.h"

#define SPK_INTERNAL __attribute__((visibility("hidden")))

#define TRY(expr)                                                                                               \
    do {                                                                                                        \
        int rc_ = (expr);                                                                                       \
        if (rc_ != SPK_OK) return rc_;                                                                          \
    } while (0)

#define RHS_CHUNK 64 /* right-hand sides per internal solve pass */

struct spike_context_s {
    int device;
    void *own_stream, *stream;
    void *copy_stream;     /* host -> device copies that overlap the factorization (created on demand) */
    void *range_streams[4]; /* the factorization of those copies' partition ranges (created on demand) */
    void *aux_stream;       /* the reduced factorization, beside the first sweep (created on demand) */
    void *range_events[9];  /* one per partition range's copy, one for the column indices (on demand) */
    /* options */
    int refs; /* the creator's reference + one per factor handle or batch using the context */
    int mode, partitions, max_refine, red_refine, timing, twist;
    int host_threads; /* SPIKE_OPT_HOST_THREADS */
    int red_fp64;     /* SPIKE_OPT_REDUCED_FP64 */
    int stream_alloc; /* workspace allocated stream-ordered on `stream` */
    double tol;
    /* cached plan for the reference-API and device-pointer calls */
    spk_plan *plan;
    int *d_scratch; /* 4 ints for the analysis kernel */
    /* staging buffers, grown on demand */
    void *d_rowptr, *d_colind, *d_aij, *d_b, *d_x, *d_r, *d_stage;
    size_t c_rowptr, c_colind, c_aij, c_b, c_x, c_r, c_stage;
    spike_info_t info;
    void *shard; /* the sharded solve's plans and buffers, kept for a next call of the same shape */
};

/* thread-local error detail (spike_last_error_code / spike_last_error) */
SPK_INTERNAL Error_t spk_fail(int code, const char *fmt, ...);
SPK_INTERNAL Error_t spk_fail_code(int spk_code, const char *where);
SPK_INTERNAL Error_t spk_succeed(void);

/* the context itself, or the calling thread's default one (created on demand) */
SPK_INTERNAL spike_context_t spk_get_ctx(spike_context_t c);
/* Handles that use a context (factors, batches) hold a reference to it, so
 * spike_context_destroy before their release only drops the creator's
 * reference: the context goes when its last handle does. */
SPK_INTERNAL void spk_ctx_ref(spike_context_t c);
SPK_INTERNAL void spk_ctx_unref(spike_context_t c);

/* smallest supported tile size >= k (0 when k is above the largest) */
SPK_INTERNAL int spk_choose_block(int k);
/* A plan for an explicit schedule: tile size KB, p partitions starting at
 * part_start[0..p] (part_start[p] = n).  Allocates the device workspace. */
SPK_INTERNAL int spk_plan_build(int n, long long nnz, int ku, int kl, int KB, int is_complex, int mode, int p,
                                const int *part_start, int nrhs_max, void *stream, int stream_alloc,
                                spk_plan **out);
/* The reduced system of p partitions (p - 1 interfaces, tile size KB) alone:
 * the arrays of spk_reduced_factor / spk_reduced_solve, nothing else. */
SPK_INTERNAL int spk_plan_reduced_build(int p, int KB, int is_complex, int mode, int nrhs_max, spk_plan **out);
/* device bytes a solve of this shape holds (plan + staging for host arrays),
 * without allocating; partitions as for spike_set_option (0 = automatic) */
SPK_INTERNAL size_t spk_solve_footprint(int n, long long nnz, int k, int nrhs, int is_complex, int mode,
                                        int partitions);
/* the reference-API solve on an explicit context (host arrays) */
SPK_INTERNAL Error_t spk_host_solve_ctx(spike_context_t c, int dtype, const char *name, integer_t n, integer_t nnz,
                                        integer_t nrhs, const integer_t *colind, const integer_t *rowptr,
                                        const void *aij, void *x, const void *b);
/* stream for workspace allocations of this context (NULL: synchronous) */
static inline void *spk_ctx_astream(spike_context_t c) { return c->stream_alloc ? c->stream : NULL; }
SPK_INTERNAL void spk_plan_destroy(spk_plan *P);
/* frees the context's sharded-solve state (spike_shard.c) */
SPK_INTERNAL void spk_shard_release(spike_context_t c);

#endif /* SPIKE_GB300_HOST_INTERNAL_H */
