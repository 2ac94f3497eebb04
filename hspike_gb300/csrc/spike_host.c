/*
 * spike_host.c -- the C host layer of libspike_gb300.so.
 *
 * Implements the reference's C API (OpenMP/spike_interfaces.h:28-72) and the
 * extensions of spike_gb300.h on top of the thin CUDA C ABI in
 * spike_internal.h.  It owns everything the reference does on the host in
 * dspike_core_host (OpenMP/spike_interfaces.c:43-419):
 *
 *   argument checks          (the reference only checks nnz < 0, :53-56)
 *   bandwidth + schedule     (spike_solve_analysis, OpenMP/spike_analysis.c:3-83)
 *   phase orchestration      factor -> reduced factor -> solve -> retrieve
 *   iterative refinement     x += SPIKE(b - A x) until ||b - A x|| / ||b||
 *                            reaches the tolerance (the reference only prints
 *                            the residual: OpenMP/spike_interfaces.c:405)
 *
 * There is no CPU compute path: every numerical step is a kernel on the
 * current CUDA device, and a missing or failing device is an error.
 */
#include <math.h>
#include <pthread.h>
#include <sched.h>
#include <stdarg.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "spike_host_internal.h"

const Error_t SPIKE_SUCCESS = 0;
const Error_t SPIKE_ERROR = 1;

/* ------------------------------------------------------------------ */
/* errors                                                               */
/* ------------------------------------------------------------------ */
static __thread int t_err_code = 0;
static __thread char t_err_msg[512] = "";

Error_t spk_fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err_msg, sizeof t_err_msg, fmt, ap);
    va_end(ap);
    t_err_code = code;
    return SPIKE_ERROR;
}

Error_t spk_fail_code(int code, const char *where)
{
    switch (code) {
    case SPK_ECUDA: return spk_fail(SPIKE_ERR_CUDA, "%s: CUDA error: %s", where, spk_cuda_error_string());
    case SPK_EMEM: return spk_fail(SPIKE_ERR_MEMORY, "%s: device allocation failed (%s)", where, spk_cuda_error_string());
    case SPK_EBAND: return spk_fail(SPIKE_ERR_BANDWIDTH, "%s: bandwidth not supported in this precision", where);
    case SPK_EPIVOT: return spk_fail(SPIKE_ERR_PIVOT, "%s: zero or non-finite pivot", where);
    case SPK_ECSR: return spk_fail(SPIKE_ERR_CSR, "%s: invalid CSR (row pointers, column range or ordering)", where);
    case SPK_ETIMEOUT:
        return spk_fail(SPIKE_ERR_CUDA, "%s: a kernel gave up waiting for a bulk copy into shared memory", where);
    default: return spk_fail(code, "%s: error %d", where, code);
    }
}

Error_t spk_succeed(void)
{
    t_err_code = SPIKE_ERR_NONE;
    t_err_msg[0] = 0;
    return SPIKE_SUCCESS;
}

int spike_last_error_code(void) { return t_err_code; }
const char *spike_last_error(void) { return t_err_msg; }

/* ------------------------------------------------------------------ */
/* contexts                                                             */
/* ------------------------------------------------------------------ */
struct spike_factor_s {
    spike_context_t ctx;
    spk_plan *plan;
    int is_complex;
    int n;
    long long nnz;
    int owns;
    const int *d_rowptr, *d_colind;
    const void *d_aij;
    void *o_rowptr, *o_colind, *o_aij; /* owned copies */
    void *d_b, *d_x, *d_r;
    size_t c_b, c_x, c_r;
    void *astream; /* allocation stream (the context's, when stream-ordered) */
    int released;
};

static __thread spike_context_t t_default = NULL;

static int ensure(void **p, size_t *cap, size_t need, void *astream)
{
    if (need <= *cap && *p) return SPK_OK;
    spk_free_on(*p, astream);
    *p = NULL;
    *cap = 0;
    TRY(spk_malloc_on(p, need, astream));
    *cap = need;
    return SPK_OK;
}


Error_t spike_context_create(spike_context_t *out)
{
    if (!out) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_context_create: NULL output");
    *out = NULL;
    if (spk_device_count() <= 0) return spk_fail(SPIKE_ERR_NO_DEVICE, "no CUDA device is visible");
    spike_context_t c = (spike_context_t)calloc(1, sizeof *c);
    if (!c) return spk_fail(SPIKE_ERR_MEMORY, "host allocation failed");
    c->device = spk_current_device();
    if (spk_stream_create(&c->own_stream) != SPK_OK) {
        free(c);
        return spk_fail_code(SPK_ECUDA, "spike_context_create");
    }
    c->stream = c->own_stream;
    c->refs = 1;
    c->mode = SPK_MIXED;
    c->partitions = 0;
    c->max_refine = 3;
    c->red_refine = 0;
    c->twist = 1;
    c->host_threads = 8;
    c->tol = 1e-12;
    if (spk_malloc((void **)&c->d_scratch, 4 * sizeof(int)) != SPK_OK) {
        spk_stream_destroy(c->own_stream);
        free(c);
        return spk_fail_code(SPK_EMEM, "spike_context_create");
    }
    *out = c;
    return spk_succeed();
}

static void ctx_free(spike_context_t c)
{
    void *as = spk_ctx_astream(c);
    spk_shard_release(c);
    spk_plan_destroy(c->plan);
    spk_free(c->d_scratch);
    spk_free_on(c->d_rowptr, as);
    spk_free_on(c->d_colind, as);
    spk_free_on(c->d_aij, as);
    spk_free_on(c->d_b, as);
    spk_free_on(c->d_x, as);
    spk_free_on(c->d_r, as);
    spk_free_on(c->d_stage, as);
    if (c->stream) spk_stream_sync(c->stream);
    spk_stream_destroy(c->own_stream);
    if (c->copy_stream) spk_stream_destroy(c->copy_stream);
    for (int i = 0; i < 4; i++)
        if (c->range_streams[i]) spk_stream_destroy(c->range_streams[i]);
    if (c->aux_stream) spk_stream_destroy(c->aux_stream);
    for (int i = 0; i < 9; i++)
        if (c->range_events[i]) spk_event_destroy(c->range_events[i]);
    if (t_default == c) t_default = NULL;
    free(c);
}

void spk_ctx_ref(spike_context_t c) { __atomic_add_fetch(&c->refs, 1, __ATOMIC_ACQ_REL); }

void spk_ctx_unref(spike_context_t c)
{
    if (__atomic_sub_fetch(&c->refs, 1, __ATOMIC_ACQ_REL) == 0) ctx_free(c);
}

Error_t spike_context_destroy(spike_context_t c)
{
    if (!c) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_context_destroy: NULL context");
    spk_ctx_unref(c);
    return spk_succeed();
}

spike_context_t spk_get_ctx(spike_context_t c)
{
    if (c) return c;
    if (!t_default && spike_context_create(&t_default) != SPIKE_SUCCESS) return NULL;
    return t_default;
}

Error_t spike_context_set_stream(spike_context_t c, void *s)
{
    c = spk_get_ctx(c);
    if (!c) return SPIKE_ERROR;
    spk_stream_sync(c->stream);
    c->stream = s ? s : c->own_stream;
    return spk_succeed();
}

Error_t spike_set_option(spike_context_t c, int opt, double v)
{
    c = spk_get_ctx(c);
    if (!c) return SPIKE_ERROR;
    switch (opt) {
    case SPIKE_OPT_PRECISION:
        if (v != SPIKE_PRECISION_MIXED && v != SPIKE_PRECISION_FP64)
            return spk_fail(SPIKE_ERR_ARGUMENT, "precision must be SPIKE_PRECISION_MIXED or SPIKE_PRECISION_FP64");
        c->mode = (v == SPIKE_PRECISION_FP64) ? SPK_PLAIN : SPK_MIXED;
        break;
    case SPIKE_OPT_PARTITIONS:
        if (v < 0 || v > 1 << 24) return spk_fail(SPIKE_ERR_ARGUMENT, "partitions must be in [0, 2^24]");
        c->partitions = (int)v;
        break;
    case SPIKE_OPT_MAX_REFINE:
        if (v < 0 || v > 100) return spk_fail(SPIKE_ERR_ARGUMENT, "max refine sweeps must be in [0, 100]");
        c->max_refine = (int)v;
        break;
    case SPIKE_OPT_TOLERANCE:
        if (!(v >= 0)) return spk_fail(SPIKE_ERR_ARGUMENT, "tolerance must be >= 0");
        c->tol = v;
        break;
    case SPIKE_OPT_REDUCED_REFINE:
        if (v < 0 || v > 20) return spk_fail(SPIKE_ERR_ARGUMENT, "reduced refine sweeps must be in [0, 20]");
        c->red_refine = (int)v;
        break;
    case SPIKE_OPT_PHASE_TIMING:
        c->timing = v != 0;
        break;
    case SPIKE_OPT_TWIST:
        c->twist = v != 0;
        break;
    case SPIKE_OPT_REDUCED_FP64:
        c->red_fp64 = v != 0;
        break;
    case SPIKE_OPT_HOST_THREADS:
        if (v < 0 || v > 64) return spk_fail(SPIKE_ERR_ARGUMENT, "host threads must be in [0, 64]");
        c->host_threads = (int)v;
        break;
    case SPIKE_OPT_STREAM_ALLOC:
        if ((v != 0) != (c->stream_alloc != 0)) {
            /* workspace changes allocator: release it (it is rebuilt on demand) */
            spk_stream_sync(c->stream);
            void *as = spk_ctx_astream(c);
            spk_plan_destroy(c->plan);
            c->plan = NULL;
            void **bufs[] = {&c->d_rowptr, &c->d_colind, &c->d_aij, &c->d_b, &c->d_x, &c->d_r, &c->d_stage};
            size_t *caps[] = {&c->c_rowptr, &c->c_colind, &c->c_aij, &c->c_b, &c->c_x, &c->c_r, &c->c_stage};
            for (int i = 0; i < 7; i++) {
                spk_free_on(*bufs[i], as);
                *bufs[i] = NULL;
                *caps[i] = 0;
            }
            spk_stream_sync(c->stream);
        }
        c->stream_alloc = v != 0;
        break;
    default: return spk_fail(SPIKE_ERR_ARGUMENT, "unknown option %d", opt);
    }
    return spk_succeed();
}

Error_t spike_get_option(spike_context_t c, int opt, double *v)
{
    c = spk_get_ctx(c);
    if (!c || !v) return c ? spk_fail(SPIKE_ERR_ARGUMENT, "NULL output") : SPIKE_ERROR;
    switch (opt) {
    case SPIKE_OPT_PRECISION: *v = c->mode == SPK_PLAIN ? SPIKE_PRECISION_FP64 : SPIKE_PRECISION_MIXED; break;
    case SPIKE_OPT_PARTITIONS: *v = c->partitions; break;
    case SPIKE_OPT_MAX_REFINE: *v = c->max_refine; break;
    case SPIKE_OPT_TOLERANCE: *v = c->tol; break;
    case SPIKE_OPT_REDUCED_REFINE: *v = c->red_refine; break;
    case SPIKE_OPT_PHASE_TIMING: *v = c->timing; break;
    case SPIKE_OPT_TWIST: *v = c->twist; break;
    case SPIKE_OPT_REDUCED_FP64: *v = c->red_fp64; break;
    case SPIKE_OPT_HOST_THREADS: *v = c->host_threads; break;
    case SPIKE_OPT_STREAM_ALLOC: *v = c->stream_alloc; break;
    default: return spk_fail(SPIKE_ERR_ARGUMENT, "unknown option %d", opt);
    }
    return spk_succeed();
}

Error_t spike_get_info(spike_context_t c, spike_info_t *info)
{
    c = spk_get_ctx(c);
    if (!c || !info) return c ? spk_fail(SPIKE_ERR_ARGUMENT, "NULL output") : SPIKE_ERROR;
    *info = c->info;
    return spk_succeed();
}

Error_t spike_get_phase_times(spike_context_t c, int nphases, double *ms, long long *calls, int reset)
{
    c = spk_get_ctx(c);
    if (!c) return SPIKE_ERROR;
    if (nphases < 0 || nphases > SPK_NPHASES) return spk_fail(SPIKE_ERR_ARGUMENT, "nphases must be in [0, %d]", SPK_NPHASES);
    spk_plan *P = c->plan;
    for (int i = 0; i < nphases; i++) {
        if (ms) ms[i] = P ? P->phase_ms[i] : 0.0;
        if (calls) calls[i] = P ? P->phase_calls[i] : 0;
    }
    if (reset && P)
        for (int i = 0; i < SPK_NPHASES; i++) {
            P->phase_ms[i] = 0.0;
            P->phase_calls[i] = 0;
        }
    return spk_succeed();
}

/* ------------------------------------------------------------------ */
/* plan: schedule + device workspace                                    */
/* ------------------------------------------------------------------ */
int spk_choose_block(int k)
{
    const int sizes[] = {2, 4, 8, 16, 32, 64, 128};
    for (int i = 0; i < 7; i++)
        if (k <= sizes[i]) return sizes[i];
    return 0;
}

/* Partition count.  The reference fixes p = 4 (OpenMP/spike_analysis.c:168)
 * and bounds it by p_max = n / (2 (ku + kl)) (:153).  Here every partition
 * must hold at least two tiles (2 KB rows) so that its top and bottom tips
 * are distinct; a requested p is clamped to that, an automatic p fills the
 * GPU: two CTAs per SM for the large tiles, more for the small ones. */
static int choose_partitions(int n, int KB, int requested)
{
    long long pmax = n / (2LL * KB);
    if (pmax < 1) pmax = 1;
    long long p = requested;
    if (p <= 0) {
        int sms = spk_sm_count();
        if (sms <= 0) sms = 152;
        const int per_sm = KB >= 128 ? 1 : KB >= 32 ? 2 : KB == 16 ? 8 : 16;
        p = (long long)sms * per_sm;
    }
    if (p > pmax) p = pmax;
    if (p < 1) p = 1;
    return (int)p;
}

void spk_plan_destroy(spk_plan *P)
{
    if (!P) return;
    spk_phase_destroy(P);
    void *ptrs[] = {P->d_part_start, P->d_blk_off, P->d_blk_part, P->d_L, P->d_G, P->d_E, P->d_V, P->d_W,
                    P->d_Bhat, P->d_T, P->d_RP, P->d_RQ, P->d_RX, P->d_RY, P->d_crP, P->d_crQ, P->d_crX, P->d_crY,
                    P->d_crM, P->d_crg, P->d_z, P->d_y, P->d_g, P->d_u, P->d_rr, P->d_du, P->d_err, P->d_norms};
    for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; i++) spk_free_on(ptrs[i], P->astream);
    free(P->part_start);
    free(P->blk_off);
    free(P->cr_count);
    free(P->cr_off);
    free(P->cr_moff);
    free(P);
}

static int palloc(spk_plan *P, void **p, size_t bytes)
{
    TRY(spk_malloc_on(p, bytes, P->astream));
    P->bytes += bytes;
    return SPK_OK;
}

/* The reduced system of p partitions alone (the arrays spk_reduced_factor and
 * spk_reduced_solve use): the interface blocks RP, RQ, RX, RY, the cyclic
 * reduction levels and the reduced right-hand side / solution.  No partition
 * is factored with it; the blocks come from elsewhere (the ranks of a sharded
 * solve). */
int spk_plan_reduced_build(int p, int KB, int is_complex, int mode, int nrhs_max, spk_plan **out)
{
    *out = NULL;
    if (p < 2 || !KB || nrhs_max < 1) return SPK_EARG;
    spk_plan *P = (spk_plan *)calloc(1, sizeof *P);
    if (!P) return SPK_EMEM;
    P->KB = KB;
    P->is_complex = is_complex;
    P->mode = mode;
    P->nrhs_max = nrhs_max;
    P->p = p;
    P->n_iface = p - 1;
    int levels = 0;
    for (int c = P->n_iface; c > 1; c = (c + 1) / 2) levels++;
    P->cr_levels = levels;
    P->cr_count = (int *)malloc(sizeof(int) * (levels + 1));
    P->cr_off = (long long *)malloc(sizeof(long long) * (levels + 2));
    P->cr_moff = (long long *)malloc(sizeof(long long) * (levels + 2));
    if (!P->cr_count || !P->cr_off || !P->cr_moff) {
        spk_plan_destroy(P);
        return SPK_EMEM;
    }
    long long tiles = 0, mtiles = 0;
    int c = P->n_iface;
    for (int l = 0; l <= levels; l++) {
        P->cr_count[l] = c;
        P->cr_off[l] = tiles;
        P->cr_moff[l] = mtiles;
        tiles += c;
        mtiles += (l < levels) ? c / 2 : 1;
        c = (c + 1) / 2;
    }
    P->cr_off[levels + 1] = tiles;
    P->cr_moff[levels + 1] = mtiles;
    P->crg_stride = tiles * 2 * KB;
    const size_t hs = (is_complex ? 2 : 1) * 8;
    const size_t TS = (size_t)KB * KB, nif = (size_t)P->n_iface;
    int rc = SPK_OK;
#define PA(ptr, bytes)                                                                                          \
    if (rc == SPK_OK) rc = palloc(P, (void **)&(ptr), (bytes))
    PA(P->d_RP, hs * TS * nif);
    PA(P->d_RQ, hs * TS * nif);
    PA(P->d_RX, hs * TS * nif);
    PA(P->d_RY, hs * TS * nif);
    PA(P->d_crP, hs * TS * tiles); /* FP64 scalars: the reduced system may run in FP64 (red_fp64) */
    PA(P->d_crQ, hs * TS * tiles);
    PA(P->d_crX, hs * TS * tiles);
    PA(P->d_crY, hs * TS * tiles);
    PA(P->d_crM, hs * TS * 4 * (mtiles > 0 ? mtiles : 1));
    PA(P->d_crg, hs * 2 * (size_t)P->crg_stride * nrhs_max);
    PA(P->d_g, hs * nif * 2 * KB * nrhs_max);
    PA(P->d_u, hs * nif * 2 * KB * nrhs_max);
    PA(P->d_rr, hs * nif * 2 * KB * nrhs_max);
    PA(P->d_du, hs * nif * 2 * KB * nrhs_max);
    PA(P->d_err, sizeof(unsigned) * 4);
#undef PA
    if (rc != SPK_OK) {
        spk_plan_destroy(P);
        return rc;
    }
    *out = P;
    return SPK_OK;
}

int spk_plan_build(int n, long long nnz, int ku, int kl, int KB, int is_complex, int mode, int p,
                   const int *part_start, int nrhs_max, void *stream, int stream_alloc, spk_plan **out)
{
    *out = NULL;
    if (!KB || spk_factor_smem(KB, is_complex, mode) == 0) return SPK_EBAND;
    spk_plan *P = (spk_plan *)calloc(1, sizeof *P);
    if (!P) return SPK_EMEM;
    P->astream = stream_alloc ? stream : NULL;
    P->n = n;
    P->nnz = nnz;
    P->ku = ku;
    P->kl = kl;
    P->KB = KB;
    P->is_complex = is_complex;
    P->mode = mode;
    P->nrhs_max = nrhs_max;
    P->p = p;
    P->n_iface = p - 1;
    P->part_start = (int *)malloc(sizeof(int) * (p + 1));
    P->blk_off = (int *)malloc(sizeof(int) * (p + 1));
    if (!P->part_start || !P->blk_off) {
        spk_plan_destroy(P);
        return SPK_EMEM;
    }
    memcpy(P->part_start, part_start, sizeof(int) * (p + 1));
    P->blk_off[0] = 0;
    for (int i = 0; i < p; i++) {
        const int m = P->part_start[i + 1] - P->part_start[i];
        P->blk_off[i + 1] = P->blk_off[i] + (m + KB - 1) / KB;
    }
    P->total_blocks = P->blk_off[p];
    P->NP = (long long)P->total_blocks * KB;
    /* two-sided partition solves pay off on long partitions (eight blocks or
     * more each, so that V's and W's right-hand sides sit in opposite halves);
     * on KB lanes per chain only while the chains are too few to fill the GPU */
    int min_blocks = 1 << 30;
    for (int i = 0; i < p; i++)
        if (P->blk_off[i + 1] - P->blk_off[i] < min_blocks) min_blocks = P->blk_off[i + 1] - P->blk_off[i];
    P->twist_cap = spk_twist_supported(KB, is_complex, mode) && min_blocks >= 8 && (KB > 4 || p <= 2048);
    P->twist = P->twist_cap;

    /* cyclic-reduction levels of the reduced system */
    int levels = 0;
    for (int c = P->n_iface; c > 1; c = (c + 1) / 2) levels++;
    P->cr_levels = levels;
    P->cr_count = (int *)malloc(sizeof(int) * (levels + 1));
    P->cr_off = (long long *)malloc(sizeof(long long) * (levels + 2));
    P->cr_moff = (long long *)malloc(sizeof(long long) * (levels + 2));
    if (!P->cr_count || !P->cr_off || !P->cr_moff) {
        spk_plan_destroy(P);
        return SPK_EMEM;
    }
    long long tiles = 0, mtiles = 0;
    int c = P->n_iface > 0 ? P->n_iface : 1;
    for (int l = 0; l <= levels; l++) {
        P->cr_count[l] = c;
        P->cr_off[l] = tiles;
        P->cr_moff[l] = mtiles;
        tiles += c;
        mtiles += (l < levels) ? c / 2 : 1;
        c = (c + 1) / 2;
    }
    P->cr_off[levels + 1] = tiles;
    P->cr_moff[levels + 1] = mtiles;
    P->crg_stride = tiles * 2 * KB;

    const size_t fs = (is_complex ? 2 : 1) * (mode == SPK_MIXED ? 4 : 8); /* factor scalar bytes */
    const size_t hs = (is_complex ? 2 : 1) * 8;                           /* FP64 scalar bytes */
    const size_t TS = (size_t)KB * KB;
    const size_t nif = P->n_iface > 0 ? (size_t)P->n_iface : 1;
    int rc = SPK_OK;
#define PA(ptr, bytes)                                                                                          \
    if (rc == SPK_OK) rc = palloc(P, (void **)&(ptr), (bytes))
    PA(P->d_part_start, sizeof(int) * (p + 1));
    PA(P->d_blk_off, sizeof(int) * (p + 1));
    PA(P->d_blk_part, sizeof(int) * P->total_blocks);
    PA(P->d_L, fs * TS * P->total_blocks);
    PA(P->d_G, fs * TS * P->total_blocks);
    PA(P->d_E, fs * TS * P->total_blocks);
    PA(P->d_W, fs * TS * P->total_blocks);
    PA(P->d_V, fs * TS * P->total_blocks);
    PA(P->d_Bhat, fs * TS * p);
    PA(P->d_T, fs * TS * 3 * P->total_blocks);
    PA(P->d_RP, hs * TS * nif);
    PA(P->d_RQ, hs * TS * nif);
    PA(P->d_RX, hs * TS * nif);
    PA(P->d_RY, hs * TS * nif);
    PA(P->d_crP, hs * TS * tiles); /* FP64 scalars: the reduced system may run in FP64 (red_fp64) */
    PA(P->d_crQ, hs * TS * tiles);
    PA(P->d_crX, hs * TS * tiles);
    PA(P->d_crY, hs * TS * tiles);
    PA(P->d_crM, hs * TS * 4 * (mtiles > 0 ? mtiles : 1));
    PA(P->d_crg, hs * 2 * (size_t)P->crg_stride * nrhs_max);
    PA(P->d_z, fs * (size_t)P->NP * nrhs_max);
    PA(P->d_y, fs * (size_t)P->NP * nrhs_max);
    PA(P->d_g, hs * nif * 2 * KB * nrhs_max);
    PA(P->d_u, hs * nif * 2 * KB * nrhs_max);
    PA(P->d_rr, hs * nif * 2 * KB * nrhs_max);
    PA(P->d_du, hs * nif * 2 * KB * nrhs_max);
    PA(P->d_err, sizeof(unsigned) * 4);
    PA(P->d_norms, sizeof(double) * 2 * nrhs_max);
#undef PA
    if (rc == SPK_OK) {
        int *bp = (int *)malloc(sizeof(int) * P->total_blocks);
        if (!bp) rc = SPK_EMEM;
        for (int i = 0; bp && i < p; i++)
            for (int b = P->blk_off[i]; b < P->blk_off[i + 1]; b++) bp[b] = i;
        if (rc == SPK_OK) rc = spk_memcpy_h2d(P->d_part_start, P->part_start, sizeof(int) * (p + 1), stream);
        if (rc == SPK_OK) rc = spk_memcpy_h2d(P->d_blk_off, P->blk_off, sizeof(int) * (p + 1), stream);
        if (rc == SPK_OK) rc = spk_memcpy_h2d(P->d_blk_part, bp, sizeof(int) * P->total_blocks, stream);
        if (rc == SPK_OK) rc = spk_stream_sync(stream);
        free(bp);
    }
    if (rc != SPK_OK) {
        spk_plan_destroy(P);
        return rc;
    }
    *out = P;
    return SPK_OK;
}

static int plan_create(int n, long long nnz, int ku, int kl, int is_complex, int mode, int partitions,
                       int nrhs_max, void *stream, int stream_alloc, spk_plan **out)
{
    *out = NULL;
    const int k = ku > kl ? ku : kl;
    const int KB = spk_choose_block(k < 1 ? 1 : k);
    if (!KB || spk_factor_smem(KB, is_complex, mode) == 0) return SPK_EBAND;
    const int p = choose_partitions(n, KB, partitions);
    int *ps = (int *)malloc(sizeof(int) * (p + 1));
    if (!ps) return SPK_EMEM;
    /* A partition count the caller asked for gets the reference's layout
     * (spike_solve_analysis: n/p rows each, the remainder in the last one);
     * a count chosen here spreads the remainder one row each over the first
     * partitions, since a long last partition's chain would set the time
     * (with many small partitions the remainder can be a hundred blocks). */
    const int nreg = n / p, rem = partitions > 0 ? 0 : n % p;
    for (int i = 0; i < p; i++) ps[i] = i * nreg + (i < rem ? i : rem);
    ps[p] = n;
    const int rc = spk_plan_build(n, nnz, ku, kl, KB, is_complex, mode, p, ps, nrhs_max, stream, stream_alloc, out);
    free(ps);
    return rc;
}

/* mirrors spk_plan_build's allocations and the staging of spk_host_solve_ctx */
size_t spk_solve_footprint(int n, long long nnz, int k, int nrhs, int is_complex, int mode, int partitions)
{
    const int KB = spk_choose_block(k < 1 ? 1 : k);
    if (!KB || n <= 0) return 0;
    const int p = choose_partitions(n, KB, partitions);
    const int nreg = n / p;
    long long blocks;
    if (partitions > 0) /* the reference's layout (plan_create) */
        blocks = (long long)(p - 1) * ((nreg + KB - 1) / KB) + ((n - (long long)(p - 1) * nreg) + KB - 1) / KB;
    else { /* balanced: n % p partitions of nreg + 1 rows */
        const int rem = n % p;
        blocks = (long long)rem * ((nreg + 1 + KB - 1) / KB) + (long long)(p - rem) * ((nreg + KB - 1) / KB);
    }
    const long long nif = p > 1 ? p - 1 : 1;
    long long tiles = 0, mtiles = 0;
    for (long long c = nif, l = 0;; l++) {
        tiles += c;
        if (c <= 1) {
            mtiles += 1;
            break;
        }
        mtiles += c / 2;
        c = (c + 1) / 2;
    }
    const int chunk = nrhs < RHS_CHUNK ? nrhs : RHS_CHUNK;
    const size_t fs = (is_complex ? 2 : 1) * (mode == SPK_MIXED ? 4 : 8);
    const size_t hs = (is_complex ? 2 : 1) * 8;
    const size_t TS = (size_t)KB * KB;
    size_t b = 0;
    b += sizeof(int) * (2 * (size_t)(p + 1) + (size_t)blocks);
    b += fs * TS * (size_t)blocks * 8 + fs * TS * p;            /* L G E W V + 3 band tiles, B^ */
    b += hs * TS * (size_t)nif * 4;                               /* RP RQ RX RY */
    b += hs * TS * (size_t)tiles * 4 + hs * TS * 4 * (size_t)mtiles; /* cyclic reduction (FP64 scalars) */
    b += hs * 2 * (size_t)tiles * 2 * KB * chunk;                 /* reduced RHS work */
    b += fs * 2 * (size_t)blocks * KB * chunk;                    /* z, y */
    b += hs * (size_t)nif * 2 * KB * chunk * 4;                   /* g u rr du */
    b += 16 + sizeof(double) * 2 * chunk;
    /* staging of a host-array solve: CSR, b, x, r */
    b += sizeof(int) * ((size_t)n + 1 + (size_t)nnz) + hs * (size_t)nnz + hs * (size_t)n * (2 * nrhs + chunk);
    return b;
}

static int plan_matches(const spk_plan *P, int n, int ku, int kl, int is_complex, int mode, int partitions, int nrhs)
{
    if (!P) return 0;
    const int k = ku > kl ? ku : kl;
    const int KB = spk_choose_block(k < 1 ? 1 : k);
    return P->n == n && P->KB == KB && P->is_complex == is_complex && P->mode == mode &&
           P->p == choose_partitions(n, KB, partitions) && nrhs <= P->nrhs_max;
}

/* ------------------------------------------------------------------ */
/* phases                                                              */
/* ------------------------------------------------------------------ */
static int check_device_error(spk_plan *P, void *stream, unsigned *e)
{
    e[0] = e[1] = e[2] = e[3] = 0;
    TRY(spk_memcpy_d2h(e, P->d_err, sizeof(unsigned) * 4, stream));
    TRY(spk_stream_sync(stream));
    if (e[0] & SPK_DEV_ERR_TIMEOUT) return SPK_ETIMEOUT;
    if (e[0] & SPK_DEV_ERR_PIVOT) return SPK_EPIVOT;
    if (e[0] & (SPK_DEV_ERR_BAND | SPK_DEV_ERR_CSR)) return SPK_ECSR;
    return SPK_OK;
}

/* The reduced factorization needs only the spikes' tips and the first
 * right-hand-side sweep y = A_i^{-1} b only the block factors: with an aux
 * stream (and no phase timing) the two run side by side, b0 being the first
 * chunk of nr0 columns.  Below OVERLAP_MIN_ROWS both are a few microseconds
 * and the fork and join would cost more than they save. */
#define OVERLAP_MIN_ROWS (1 << 18)
static int reduced_and_first_sweep(spk_plan *P, void *stream, void *aux, const void *b0, int nr0)
{
    P->first_applied = 0;
    if (aux && b0 && nr0 > 0 && !P->timing && P->n >= OVERLAP_MIN_ROWS) {
        TRY(spk_stream_fork(stream, aux));
        TRY(spk_reduced_factor(P, aux));
        TRY(spk_apply(P, b0, nr0, stream));
        TRY(spk_stream_fork(aux, stream));
        P->first_applied = 1;
        return SPK_OK;
    }
    spk_phase_begin(P, SPK_PH_RED_FACTOR, stream);
    TRY(spk_reduced_factor(P, stream));
    spk_phase_end(P, stream);
    return SPK_OK;
}

/* e (optional): the device error word and, with P->validate, ku and kl */
static int factor_phase_e(spk_plan *P, const int *rp, const int *ci, const void *aij, void *stream, unsigned *e,
                          void *aux, const void *b0, int nr0)
{
    unsigned w[4];
    TRY(spk_memset(P->d_err, 0, sizeof(unsigned) * 4, stream));
    TRY(spk_factor(P, rp, ci, aij, stream));
    TRY(reduced_and_first_sweep(P, stream, aux, b0, nr0));
    return check_device_error(P, stream, e ? e : w);
}

static int factor_phase(spk_plan *P, const int *rp, const int *ci, const void *aij, void *stream)
{
    return factor_phase_e(P, rp, ci, aij, stream, NULL, NULL, NULL, 0);
}

/* one SPIKE application: x (+)= A_spike^{-1} r */
static int spike_apply_once(spk_plan *P, void *x, const void *r, int nrhs, int red, int accumulate, void *stream)
{
    if (P->first_applied) {
        P->first_applied = 0; /* y = A_i^{-1} r ran beside the reduced factorization */
    } else {
        spk_phase_begin(P, SPK_PH_APPLY, stream);
        TRY(spk_apply(P, r, nrhs, stream));
        spk_phase_end(P, stream);
    }
    spk_phase_begin(P, SPK_PH_RED_SOLVE, stream);
    TRY(spk_reduced_solve(P, nrhs, red, stream));
    spk_phase_end(P, stream);
    spk_phase_begin(P, SPK_PH_RETRIEVE, stream);
    TRY(spk_retrieve(P, x, nrhs, accumulate, stream));
    spk_phase_end(P, stream);
    return SPK_OK;
}

typedef struct {
    int max_refine, red_refine;
    double tol;
    double relres_max;
    int sweeps;
} refine_opts;

/* x = A^{-1} b for nrhs <= P->nrhs_max columns, refined in FP64. */
static int solve_phase(spk_plan *P, const int *rp, const int *ci, const void *aij, void *x, const void *b, void *r,
                       int nrhs, refine_opts *o, void *stream)
{
    const int red = o->red_refine > 0 ? o->red_refine : (P->mode == SPK_MIXED && !P->red_fp64 ? 2 : 1);
    double norms[2 * RHS_CHUNK];
    double bnorm[RHS_CHUNK];
    TRY(spike_apply_once(P, x, b, nrhs, red, 0, stream));
    for (int sweep = 0;; sweep++) {
        spk_phase_begin(P, SPK_PH_RESIDUAL, stream);
        TRY(spk_residual(P, rp, ci, aij, x, b, r, nrhs, sweep == 0, P->d_norms, stream));
        spk_phase_end(P, stream);
        TRY(spk_memcpy_d2h(norms, P->d_norms, sizeof(double) * 2 * nrhs, stream));
        TRY(spk_stream_sync(stream));
        double worst = 0.0;
        for (int h = 0; h < nrhs; h++) {
            if (sweep == 0) bnorm[h] = sqrt(norms[nrhs + h]);
            const double rel = sqrt(norms[h]) / (bnorm[h] > 0 ? bnorm[h] : 1.0);
            if (!(rel <= worst)) worst = rel; /* NaN propagates */
        }
        o->relres_max = worst;
        o->sweeps = sweep;
        if (worst <= o->tol) return SPK_OK;
        if (sweep >= o->max_refine) return SPK_ECONV;
        TRY(spike_apply_once(P, x, r, nrhs, red, 1, stream));
    }
}

/* solve all columns in chunks of P->nrhs_max */
static int solve_all(spk_plan *P, const int *rp, const int *ci, const void *aij, void *x, const void *b, void *r,
                     int nrhs, refine_opts *o, void *stream)
{
    const size_t hs = (P->is_complex ? 2 : 1) * 8;
    double worst = 0.0;
    int sweeps = 0, rc = SPK_OK;
    for (int h0 = 0; h0 < nrhs; h0 += P->nrhs_max) {
        const int nr = nrhs - h0 < P->nrhs_max ? nrhs - h0 : P->nrhs_max;
        refine_opts oc = *o;
        const size_t off = (size_t)h0 * P->n * hs;
        rc = solve_phase(P, rp, ci, aij, (char *)x + off, (const char *)b + off, r, nr, &oc, stream);
        if (!(oc.relres_max <= worst)) worst = oc.relres_max;
        if (oc.sweeps > sweeps) sweeps = oc.sweeps;
        if (rc != SPK_OK && rc != SPK_ECONV) return rc;
        if (rc == SPK_ECONV) break;
    }
    o->relres_max = worst;
    o->sweeps = sweeps;
    return rc;
}

static void fill_info(spike_context_t c, const spk_plan *P, const refine_opts *o, long long launches)
{
    c->info.relres_max = o->relres_max;
    c->info.refine_sweeps = o->sweeps;
    c->info.partitions = P->p;
    c->info.ku = P->ku;
    c->info.kl = P->kl;
    c->info.block = P->KB;
    c->info.kernel_launches = launches;
    c->info.device_bytes = P->bytes;
    c->info.twisted = P->twist;
    c->info.columns_implied = P->impl_cols;
    c->info.reduced_fp64 = P->red_fp64 || P->mode == SPK_PLAIN;
}

static Error_t finish(int rc, const char *where, const refine_opts *o)
{
    if (rc == SPK_OK) return spk_succeed();
    if (rc == SPK_ECONV)
        return spk_fail(SPIKE_ERR_CONVERGENCE, "%s: relative residual %.3e above tolerance %.3e after %d sweeps", where,
                    o->relres_max, o->tol, o->sweeps);
    if (rc == SPK_ECSR) return spk_fail(SPIKE_ERR_CSR, "%s: invalid CSR (row pointers, column range or ordering)", where);
    return spk_fail_code(rc, where);
}

/* analysis + plan + factor + solve on device-resident FP64 data */
static int run_device(spike_context_t c, int n, long long nnz, int nrhs, const int *rp, const int *ci,
                      const void *aij, void *x, const void *b, int is_complex, refine_opts *o, long long *launches)
{
    int info[3];
    long long l0 = 0;
    const int chunk0 = nrhs < RHS_CHUNK ? nrhs : RHS_CHUNK;
    const size_t hs0 = (is_complex ? 2 : 1) * 8;
    /* A call with the shape of the previous one (n, nnz, precision,
     * partitions) reuses its plan without the separate analysis pass: the
     * band-tile pass validates the CSR and measures the bandwidth itself, and
     * only if the bandwidth class changed (or the CSR is invalid) does the
     * call fall back to analysis, a new plan and a second factorization. */
    spk_plan *Q = c->plan;
    if (Q && Q->n == n && Q->nnz == nnz && Q->is_complex == is_complex && Q->mode == c->mode &&
        Q->p == choose_partitions(n, Q->KB, c->partitions) && chunk0 <= Q->nrhs_max) {
        unsigned e[4];
        Q->twist = Q->twist_cap && c->twist;
        Q->red_fp64 = c->red_fp64 && Q->KB <= 64;
        Q->launches = 0;
        Q->timing = c->timing;
        Q->validate = 1;
        TRY(ensure(&c->d_r, &c->c_r, hs0 * (size_t)n * chunk0, spk_ctx_astream(c)));
        if (!c->aux_stream && n >= OVERLAP_MIN_ROWS) TRY(spk_stream_create(&c->aux_stream));
        const int frc = factor_phase_e(Q, rp, ci, aij, c->stream, e, c->aux_stream, b,
                                       nrhs < Q->nrhs_max ? nrhs : Q->nrhs_max);
        Q->validate = 0;
        const int ku = (int)e[1], kl = (int)e[2], kmax = ku > kl ? ku : kl;
        const int same = !(e[0] & (SPK_DEV_ERR_CSR | SPK_DEV_ERR_BAND)) && spk_choose_block(kmax < 1 ? 1 : kmax) == Q->KB;
        if (same && (frc == SPK_OK || frc == SPK_EPIVOT)) {
            Q->ku = ku;
            Q->kl = kl;
            int rc = frc;
            if (rc == SPK_OK) rc = solve_all(Q, rp, ci, aij, x, b, c->d_r, nrhs, o, c->stream);
            Q->first_applied = 0;
            if (Q->timing && (rc == SPK_OK || rc == SPK_ECONV) && spk_phase_collect(Q) != SPK_OK) rc = SPK_ECUDA;
            *launches = Q->launches;
            fill_info(c, Q, o, Q->launches);
            return rc;
        }
        Q->first_applied = 0;
        if (frc != SPK_OK && frc != SPK_ECSR && frc != SPK_EPIVOT) return frc;
        /* otherwise: the full path below */
    }
    /* the analysis is timed on the previous call's plan (the plan for this
     * call depends on its result) */
    spk_plan *Pa = c->timing ? c->plan : NULL;
    if (Pa) {
        Pa->timing = 1;
        spk_phase_begin(Pa, SPK_PH_ANALYZE, c->stream);
    }
    const int arc = spk_analyze(n, nnz, rp, ci, c->d_scratch, info, c->stream, &l0);
    if (Pa) spk_phase_end(Pa, c->stream);
    TRY(arc);
    if (info[2]) return SPK_ECSR;
    const int chunk = nrhs < RHS_CHUNK ? nrhs : RHS_CHUNK;
    if (!plan_matches(c->plan, n, info[0], info[1], is_complex, c->mode, c->partitions, chunk)) {
        spk_plan_destroy(c->plan);
        c->plan = NULL;
        TRY(plan_create(n, nnz, info[0], info[1], is_complex, c->mode, c->partitions, chunk, c->stream, c->stream_alloc,
                        &c->plan));
    }
    spk_plan *P = c->plan;
    P->nnz = nnz;
    P->ku = info[0];
    P->kl = info[1];
    P->twist = P->twist_cap && c->twist;
    P->red_fp64 = c->red_fp64 && P->KB <= 64;
    P->launches = l0;
    P->timing = c->timing;
    const size_t hs = (is_complex ? 2 : 1) * 8;
    TRY(ensure(&c->d_r, &c->c_r, hs * (size_t)n * chunk, spk_ctx_astream(c)));
    if (!c->aux_stream && n >= OVERLAP_MIN_ROWS) TRY(spk_stream_create(&c->aux_stream));
    int rc = factor_phase_e(P, rp, ci, aij, c->stream, NULL, c->aux_stream, b,
                            nrhs < P->nrhs_max ? nrhs : P->nrhs_max);
    if (rc == SPK_OK) rc = solve_all(P, rp, ci, aij, x, b, c->d_r, nrhs, o, c->stream);
    P->first_applied = 0;
    if (P->timing && (rc == SPK_OK || rc == SPK_ECONV) && spk_phase_collect(P) != SPK_OK) rc = SPK_ECUDA;
    *launches = P->launches;
    fill_info(c, P, o, P->launches);
    return rc;
}

static void opts_from(const spike_context_t c, refine_opts *o)
{
    o->max_refine = c->max_refine;
    o->red_refine = c->red_refine;
    o->tol = c->tol;
    o->relres_max = 0;
    o->sweeps = 0;
}

/* ------------------------------------------------------------------ */
/* reference API: host arrays                                           */
/* ------------------------------------------------------------------ */
static Error_t host_solve(int dtype, const char *name, integer_t n, integer_t nnz, integer_t nrhs,
                          const integer_t *colind, const integer_t *rowptr, const void *aij, void *x, const void *b)
{
    if (n < 0 || nnz < 0 || nrhs < 0) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: n, nnz and nrhs must be >= 0", name);
    if (n == 0 || nrhs == 0) return spk_succeed();
    if (!colind || !rowptr || !aij || !x || !b) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: NULL array", name);
    spike_context_t c = spk_get_ctx(NULL);
    if (!c) return SPIKE_ERROR;
    return spk_host_solve_ctx(c, dtype, name, n, nnz, nrhs, colind, rowptr, aij, x, b);
}

static Error_t solve_on(spike_context_t c, int dtype, const char *name, integer_t n, integer_t nnz, integer_t nrhs,
                        const integer_t *colind, const integer_t *rowptr, const void *aij, void *x, const void *b)
{
    if (n < 0 || nnz < 0 || nrhs < 0) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: n, nnz and nrhs must be >= 0", name);
    if (n == 0 || nrhs == 0) return spk_succeed();
    if (!colind || !rowptr || !aij || !x || !b) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: NULL array", name);
    c = spk_get_ctx(c);
    if (!c) return SPIKE_ERROR;
    return spk_host_solve_ctx(c, dtype, name, n, nnz, nrhs, colind, rowptr, aij, x, b);
}

Error_t spike_dsolve(spike_context_t ctx, integer_t n, integer_t nnz, integer_t nrhs, const integer_t *colind,
                     const integer_t *rowptr, const double *aij, double *x, const double *b)
{
    return solve_on(ctx, SPK_D, "spike_dsolve", n, nnz, nrhs, colind, rowptr, aij, x, b);
}

Error_t spike_zsolve(spike_context_t ctx, integer_t n, integer_t nnz, integer_t nrhs, const integer_t *colind,
                     const integer_t *rowptr, const void *aij, void *x, const void *b)
{
    return solve_on(ctx, SPK_Z, "spike_zsolve", n, nnz, nrhs, colind, rowptr, aij, x, b);
}

/* ---- the full-band check of a host CSR, on worker threads ----
 * A call with host arrays sends the matrix over the host link, the larger
 * part of its time.  When every row r holds exactly the columns
 * max(0, r - kl) .. min(n - 1, r + ku) -- the full band of the plan's ku, kl,
 * as the reference's own banded systems are stored -- the column indices
 * follow from the row pointers, so only the values need to travel: worker
 * threads check the rows range by range while the values' copies run, and
 * each range's kernels start once its rows have passed.  The first range
 * that fails sends the column indices after all and finishes on the general
 * path (the band tiles then validate it on the device). */
#define PIPE_RANGES 8
#define SCAN_MAX_THREADS 64

typedef struct {
    const int *rowptr, *colind;
    int n, ku, kl, nthreads;
    long long nnz;
    int row_lo[PIPE_RANGES + 1];
    atomic_int done[PIPE_RANGES]; /* workers finished with range g */
    atomic_int bad[PIPE_RANGES];  /* a row of range g is not the full band */
    atomic_int stop;              /* no further rows need checking */
} band_scan;

typedef struct {
    band_scan *S;
    int id;
} band_scan_arg;

/* 16-byte generic vectors (GCC's vector extension, no target intrinsics):
 * the check streams host memory, and scalar code would bind it to the core */
typedef int spk_v4i __attribute__((vector_size(16)));

static int rows_full_band(const band_scan *S, int r0, int r1)
{
    const int n = S->n, ku = S->ku, kl = S->kl;
    const spk_v4i step = {8, 8, 8, 8};
    for (int r = r0; r < r1; r++) {
        const long long lo = (long long)r - kl, hi = (long long)r + ku; /* any ku, kl: no int overflow */
        const int c0 = lo < 0 ? 0 : (int)lo, c1 = hi > n - 1 ? n - 1 : (int)hi, len = c1 - c0 + 1;
        const long long t0 = S->rowptr[r], t1 = S->rowptr[r + 1];
        if (t0 < 0 || t1 > S->nnz || t1 - t0 != (long long)len) return 0;
        const int *ci = S->colind + t0;
        spk_v4i ia = {c0, c0 + 1, c0 + 2, c0 + 3}, ib = ia + 4, da = {0, 0, 0, 0}, db = da;
        int t = 0;
        for (; t + 8 <= len; t += 8) {
            spk_v4i va, vb;
            memcpy(&va, ci + t, sizeof va);
            memcpy(&vb, ci + t + 4, sizeof vb);
            da |= va ^ ia;
            db |= vb ^ ib;
            ia += step;
            ib += step;
        }
        da |= db;
        int diff = da[0] | da[1] | da[2] | da[3];
        for (; t < len; t++) diff |= ci[t] ^ (c0 + t);
        if (diff) return 0;
    }
    return 1;
}

Error_t spike_csr_full_band(integer_t n, integer_t nnz, integer_t ku, integer_t kl, const integer_t *colind,
                            const integer_t *rowptr, int *full)
{
    if (n < 0 || nnz < 0 || ku < 0 || kl < 0 || !full || (n > 0 && !rowptr) || (nnz > 0 && !colind))
        return spk_fail(SPIKE_ERR_ARGUMENT, "spike_csr_full_band: bad argument");
    band_scan S;
    S.rowptr = rowptr;
    S.colind = colind;
    S.n = n;
    S.ku = ku;
    S.kl = kl;
    S.nnz = nnz;
    *full = n == 0 ? nnz == 0 : rowptr[0] == 0 && rowptr[n] == nnz && rows_full_band(&S, 0, n);
    return spk_succeed();
}

static void *band_scan_worker(void *p)
{
    const band_scan_arg *a = (const band_scan_arg *)p;
    band_scan *S = a->S;
    for (int g = 0; g < PIPE_RANGES; g++) {
        if (!atomic_load(&S->stop)) {
            const long long lo = S->row_lo[g], len = S->row_lo[g + 1] - lo;
            const int r0 = (int)(lo + len * a->id / S->nthreads), r1 = (int)(lo + len * (a->id + 1) / S->nthreads);
            if (!rows_full_band(S, r0, r1)) {
                atomic_store(&S->bad[g], 1); /* before stop: a range skipped after it counts as unchecked */
                atomic_store(&S->stop, 1);
            }
        }
        atomic_fetch_add(&S->done[g], 1);
    }
    return NULL;
}

/* Host arrays, plan reused (same shape as the previous call on the context)
 * and two-sided: the matrix goes to the device in partition ranges on a copy
 * stream, and each range's band tiles and chains start as soon as its rows
 * have arrived, so the factorization hides behind the copy (host -> device
 * copies are the larger part of such a call).  With host threads the column
 * indices stay on the host when the rows are the full band (above).  Returns
 * SPK_EARG when the path does not apply; the caller then copies everything
 * and solves. */
static int host_pipelined(spike_context_t c, int n, long long nnz, int nrhs, const int *colind, const int *rowptr,
                          const void *aij, const void *b, int cplx, refine_opts *o, long long *launches)
{
    spk_plan *Q = c->plan;
    const int chunk = nrhs < RHS_CHUNK ? nrhs : RHS_CHUNK;
    if (!Q || Q->n != n || Q->nnz != nnz || Q->is_complex != cplx || Q->mode != c->mode || !Q->twist_cap || !c->twist ||
        Q->p != choose_partitions(n, Q->KB, c->partitions) || chunk > Q->nrhs_max || Q->p < PIPE_RANGES ||
        Q->KB < 16 || Q->KB > 64 ||
        nnz < (8LL << 20) || c->timing)
        return SPK_EARG;
    /* the ranges' entry bounds come from the caller's row pointers */
    long long tb[PIPE_RANGES + 1];
    for (int r = 0; r <= PIPE_RANGES; r++) {
        const int prt = (int)((long long)Q->p * r / PIPE_RANGES);
        tb[r] = rowptr[Q->part_start[prt]];
        if (tb[r] < 0 || tb[r] > nnz || (r > 0 && tb[r] < tb[r - 1])) return SPK_EARG;
    }
    if (tb[0] != 0 || tb[PIPE_RANGES] != nnz) return SPK_EARG;
    const size_t hs = (cplx ? 2 : 1) * 8;
    if (!c->copy_stream) TRY(spk_stream_create(&c->copy_stream));
    for (int i = 0; i < 4; i++)
        if (!c->range_streams[i]) TRY(spk_stream_create(&c->range_streams[i]));
    for (int i = 0; i <= PIPE_RANGES; i++)
        if (!c->range_events[i]) TRY(spk_event_create(&c->range_events[i]));
    void *cs = c->copy_stream;
    void **ev = c->range_events; /* ev[r]: range r's entries are on the device; ev[PIPE_RANGES]: all columns */
    TRY(spk_stream_fork(c->stream, cs)); /* after whatever the caller queued on the context's stream */
    TRY(spk_memcpy_h2d(c->d_rowptr, rowptr, sizeof(int) * ((size_t)n + 1), cs));
    TRY(spk_memcpy_h2d(c->d_b, b, hs * (size_t)n * nrhs, cs));
    TRY(ensure(&c->d_r, &c->c_r, hs * (size_t)n * chunk, spk_ctx_astream(c)));
    Q->twist = 1;
    Q->red_fp64 = c->red_fp64 && Q->KB <= 64;
    Q->launches = 0;
    Q->timing = 0;
    Q->validate = 1;
    Q->impl_cols = 0;
    Q->impl_kl = Q->kl;
    int rc = spk_memset(Q->d_err, 0, sizeof(unsigned) * 4, c->stream);
    if (rc == SPK_OK) rc = spk_stream_fork(c->stream, cs); /* the cleared error word before any range */

    /* the band check's workers (none: copy the columns with the values) */
    band_scan S;
    pthread_t th[SCAN_MAX_THREADS];
    band_scan_arg args[SCAN_MAX_THREADS];
    int workers = 0;
    int implied = 0; /* ranges so far have implied columns */
    if (rc == SPK_OK && c->host_threads > 0 && rowptr[0] == 0) {
        const int want = c->host_threads < SCAN_MAX_THREADS ? c->host_threads : SCAN_MAX_THREADS;
        S.rowptr = rowptr;
        S.colind = colind;
        S.n = n;
        S.ku = Q->ku;
        S.kl = Q->kl;
        S.nnz = nnz;
        S.nthreads = want;
        for (int r = 0; r <= PIPE_RANGES; r++) S.row_lo[r] = Q->part_start[(int)((long long)Q->p * r / PIPE_RANGES)];
        for (int g = 0; g < PIPE_RANGES; g++) {
            atomic_init(&S.done[g], 0);
            atomic_init(&S.bad[g], 0);
        }
        atomic_init(&S.stop, 0);
        for (int i = 0; i < want; i++) {
            args[i].S = &S;
            args[i].id = i;
            if (pthread_create(&th[i], NULL, band_scan_worker, &args[i]) != 0) break;
            workers++;
        }
        if (workers < want) { /* the rows are split among `want`: without all of them, copy the columns */
            atomic_store(&S.stop, 1);
            for (int i = 0; i < workers; i++) pthread_join(th[i], NULL);
            workers = 0;
        }
        implied = workers > 0;
    }
    int columns_sent = 0; /* every column index is (or will be, on cs) on the device */
    if (implied) { /* the values first, all of them: their copies are what the check hides behind */
        for (int r = 0; r < PIPE_RANGES && rc == SPK_OK; r++) {
            const size_t e0 = (size_t)tb[r], ne = (size_t)(tb[r + 1] - tb[r]);
            if (ne) rc = spk_memcpy_h2d((char *)c->d_aij + hs * e0, (const char *)aij + hs * e0, hs * ne, cs);
            if (rc == SPK_OK) rc = spk_event_record(ev[r], cs);
        }
    }
    const int all_tried = implied;
    int all_implied = implied;
    int late = 0; /* the column indices follow every value (a range failed the check) */
    int n_implied = 0; /* ranges factored with implied columns */
    /* ranges are factored on a few streams at once: one range's chains use a
     * fraction of the GPU */
    for (int r = 0; r < PIPE_RANGES && rc == SPK_OK; r++) {
        const int p0 = (int)((long long)Q->p * r / PIPE_RANGES), p1 = (int)((long long)Q->p * (r + 1) / PIPE_RANGES);
        const size_t e0 = (size_t)tb[r], ne = (size_t)(tb[r + 1] - tb[r]);
        void *rs = c->range_streams[r % 4];
        if (implied) {
            while (atomic_load(&S.done[r]) < workers) sched_yield();
            if (atomic_load(&S.bad[r])) { /* from this range on: the columns go over as well */
                implied = 0;
                all_implied = 0;
                late = 1;
                rc = spk_memcpy_h2d(c->d_colind, colind, sizeof(int) * (size_t)nnz, cs);
                if (rc == SPK_OK) rc = spk_event_record(ev[PIPE_RANGES], cs);
                columns_sent = 1;
            }
        } else if (!all_tried) { /* no check: each range's columns and values together */
            if (ne) {
                rc = spk_memcpy_h2d((int *)c->d_colind + e0, colind + e0, sizeof(int) * ne, cs);
                if (rc == SPK_OK)
                    rc = spk_memcpy_h2d((char *)c->d_aij + hs * e0, (const char *)aij + hs * e0, hs * ne, cs);
            }
            if (rc == SPK_OK) rc = spk_event_record(ev[r], cs);
            if (r == PIPE_RANGES - 1) columns_sent = 1;
        }
        if (rc == SPK_OK) rc = spk_stream_wait_event(rs, late ? ev[PIPE_RANGES] : ev[r]);
        if (rc == SPK_OK) {
            Q->impl_cols = implied;
            n_implied += implied;
            rc = spk_factor_range(Q, (const int *)c->d_rowptr, (const int *)c->d_colind, c->d_aij, p0, p1, rs);
        }
    }
    if (workers) {
        atomic_store(&S.stop, 1);
        for (int i = 0; i < workers; i++) pthread_join(th[i], NULL);
    }
    Q->impl_cols = all_implied; /* the residual reads columns unless every range had them implied */
    for (int i = 0; i < 4 && rc == SPK_OK; i++) rc = spk_stream_fork(c->range_streams[i], c->stream);
    if (rc == SPK_OK) rc = spk_stream_fork(cs, c->stream);
    if (rc == SPK_OK) rc = spk_factor_tips(Q, c->stream);
    if (rc == SPK_OK && !c->aux_stream) rc = spk_stream_create(&c->aux_stream);
    if (rc == SPK_OK)
        rc = reduced_and_first_sweep(Q, c->stream, c->aux_stream, c->d_b, nrhs < Q->nrhs_max ? nrhs : Q->nrhs_max);
    Q->validate = 0;
    unsigned e[4] = {0, 0, 0, 0};
    if (rc == SPK_OK) {
        const int frc = check_device_error(Q, c->stream, e);
        /* ranges with implied columns are the plan's band exactly; the others measured theirs */
        int ku = (int)e[1], kl = (int)e[2];
        if (n_implied) {
            if (Q->ku > ku) ku = Q->ku;
            if (Q->kl > kl) kl = Q->kl;
        }
        const int kmax = ku > kl ? ku : kl;
        const int same =
            !(e[0] & (SPK_DEV_ERR_CSR | SPK_DEV_ERR_BAND)) && spk_choose_block(kmax < 1 ? 1 : kmax) == Q->KB;
        if (!same) {
            Q->first_applied = 0;
            Q->impl_cols = 0;
            /* the general path re-plans with the whole matrix on the device */
            if (!columns_sent) rc = spk_memcpy_h2d(c->d_colind, colind, sizeof(int) * (size_t)nnz, c->stream);
            long long l2 = 0;
            if (rc == SPK_OK)
                rc = run_device(c, n, nnz, nrhs, (const int *)c->d_rowptr, (const int *)c->d_colind, c->d_aij,
                                c->d_x, c->d_b, cplx, o, &l2);
            *launches = Q->launches + l2;
            return rc;
        }
        Q->ku = ku;
        Q->kl = kl;
        rc = frc;
    }
    if (rc == SPK_OK)
        rc = solve_all(Q, (const int *)c->d_rowptr, (const int *)c->d_colind, c->d_aij, c->d_x, c->d_b, c->d_r, nrhs, o,
                       c->stream);
    Q->first_applied = 0;
    *launches = Q->launches;
    fill_info(c, Q, o, Q->launches);
    Q->impl_cols = 0;
    return rc;
}

Error_t spk_host_solve_ctx(spike_context_t c, int dtype, const char *name, integer_t n, integer_t nnz, integer_t nrhs,
                           const integer_t *colind, const integer_t *rowptr, const void *aij, void *x, const void *b)
{
    if (n == 0 || nrhs == 0) return spk_succeed();
    const int cplx = dtype == SPK_C || dtype == SPK_Z;
    const int wide = dtype == SPK_S || dtype == SPK_C;
    const size_t es = (cplx ? 2 : 1) * (wide ? 4 : 8); /* caller element bytes */
    const size_t hs = (cplx ? 2 : 1) * 8;
    const size_t nb = (size_t)n * nrhs;
    refine_opts o;
    opts_from(c, &o);
    int rc = SPK_OK;
    rc = ensure(&c->d_rowptr, &c->c_rowptr, sizeof(int) * ((size_t)n + 1), spk_ctx_astream(c));
    if (rc == SPK_OK) rc = ensure(&c->d_colind, &c->c_colind, sizeof(int) * (size_t)(nnz ? nnz : 1), spk_ctx_astream(c));
    if (rc == SPK_OK) rc = ensure(&c->d_aij, &c->c_aij, hs * (size_t)(nnz ? nnz : 1), spk_ctx_astream(c));
    if (rc == SPK_OK) rc = ensure(&c->d_b, &c->c_b, hs * nb, spk_ctx_astream(c));
    if (rc == SPK_OK) rc = ensure(&c->d_x, &c->c_x, hs * nb, spk_ctx_astream(c));
    if (rc == SPK_OK && wide) {
        const size_t m = (size_t)nnz > nb ? (size_t)nnz : nb;
        rc = ensure(&c->d_stage, &c->c_stage, es * (m ? m : 1), spk_ctx_astream(c));
    }
    if (rc != SPK_OK) return finish(rc, name, &o);
    long long launches = 0;
    if (!wide) {
        long long lp = 0;
        rc = host_pipelined(c, n, nnz, nrhs, colind, rowptr, aij, b, cplx, &o, &lp);
        if (rc != SPK_EARG) { /* the pipelined path ran (to success or a real error) */
            launches += lp;
            if (rc == SPK_OK || rc == SPK_ECONV) {
                int rc2 = spk_memcpy_d2h(x, c->d_x, es * nb, c->stream);
                if (rc2 == SPK_OK) rc2 = spk_stream_sync(c->stream);
                if (rc2 != SPK_OK) rc = rc2;
            } else {
                spk_stream_sync(c->stream);
            }
            c->info.kernel_launches = launches;
            return finish(rc, name, &o);
        }
        rc = SPK_OK;
    }
    rc = spk_memcpy_h2d(c->d_rowptr, rowptr, sizeof(int) * ((size_t)n + 1), c->stream);
    if (rc == SPK_OK && nnz) rc = spk_memcpy_h2d(c->d_colind, colind, sizeof(int) * (size_t)nnz, c->stream);
    if (wide) {
        if (rc == SPK_OK && nnz) rc = spk_memcpy_h2d(c->d_stage, aij, es * (size_t)nnz, c->stream);
        if (rc == SPK_OK) rc = spk_widen(c->d_stage, c->d_aij, nnz, cplx, c->stream, &launches);
        if (rc == SPK_OK) rc = spk_memcpy_h2d(c->d_stage, b, es * nb, c->stream);
        if (rc == SPK_OK) rc = spk_widen(c->d_stage, c->d_b, (long long)nb, cplx, c->stream, &launches);
    } else {
        if (rc == SPK_OK && nnz) rc = spk_memcpy_h2d(c->d_aij, aij, es * (size_t)nnz, c->stream);
        if (rc == SPK_OK) rc = spk_memcpy_h2d(c->d_b, b, es * nb, c->stream);
    }
    long long l2 = 0;
    if (rc == SPK_OK)
        rc = run_device(c, n, nnz, nrhs, (const int *)c->d_rowptr, (const int *)c->d_colind, c->d_aij, c->d_x, c->d_b,
                        cplx, &o, &l2);
    launches += l2;
    /* x is written back after a convergence shortfall too (it is the last iterate) */
    if (rc == SPK_OK || rc == SPK_ECONV) {
        int rc2 = SPK_OK;
        if (wide) {
            rc2 = spk_narrow(c->d_x, c->d_stage, (long long)nb, cplx, c->stream, &launches);
            if (rc2 == SPK_OK) rc2 = spk_memcpy_d2h(x, c->d_stage, es * nb, c->stream);
        } else {
            rc2 = spk_memcpy_d2h(x, c->d_x, es * nb, c->stream);
        }
        if (rc2 == SPK_OK) rc2 = spk_stream_sync(c->stream);
        if (rc2 != SPK_OK) rc = rc2;
    } else {
        spk_stream_sync(c->stream);
    }
    c->info.kernel_launches = launches;
    return finish(rc, name, &o);
}

Error_t sspike_core_host(const integer_t n, const integer_t nnz, const integer_t nrhs, integer_t *colind,
                         integer_t *rowptr, float *aij, float *xij, float *bij)
{
    return host_solve(SPK_S, "sspike_core_host", n, nnz, nrhs, colind, rowptr, aij, xij, bij);
}
Error_t dspike_core_host(const integer_t n, const integer_t nnz, const integer_t nrhs, integer_t *colind,
                         integer_t *rowptr, double *aij, double *xij, double *bij)
{
    return host_solve(SPK_D, "dspike_core_host", n, nnz, nrhs, colind, rowptr, aij, xij, bij);
}
Error_t cspike_core_host(const integer_t n, const integer_t nnz, const integer_t nrhs, integer_t *colind,
                         integer_t *rowptr, complex8 *aij, complex8 *xij, complex8 *bij)
{
    return host_solve(SPK_C, "cspike_core_host", n, nnz, nrhs, colind, rowptr, aij, xij, bij);
}
Error_t zspike_core_host(const integer_t n, const integer_t nnz, const integer_t nrhs, integer_t *colind,
                         integer_t *rowptr, complex16 *aij, complex16 *xij, complex16 *bij)
{
    return host_solve(SPK_Z, "zspike_core_host", n, nnz, nrhs, colind, rowptr, aij, xij, bij);
}
Error_t dspike_core_host_blocking(const integer_t n, const integer_t nnz, const integer_t nrhs, integer_t *colind,
                                  integer_t *rowptr, double *aij, double *xij, double *bij)
{
    return host_solve(SPK_D, "dspike_core_host_blocking", n, nnz, nrhs, colind, rowptr, aij, xij, bij);
}

/* ------------------------------------------------------------------ */
/* device-pointer API                                                   */
/* ------------------------------------------------------------------ */
static Error_t device_solve(spike_context_t c, int cplx, const char *name, integer_t n, integer_t nnz, integer_t nrhs,
                            const integer_t *ci, const integer_t *rp, const void *aij, void *x, const void *b)
{
    if (n < 0 || nnz < 0 || nrhs < 0) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: n, nnz and nrhs must be >= 0", name);
    if (n == 0 || nrhs == 0) return spk_succeed();
    if (!ci || !rp || !aij || !x || !b) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: NULL array", name);
    c = spk_get_ctx(c);
    if (!c) return SPIKE_ERROR;
    refine_opts o;
    opts_from(c, &o);
    long long launches = 0;
    int rc = run_device(c, n, nnz, nrhs, rp, ci, aij, x, b, cplx, &o, &launches);
    if (rc != SPK_OK) spk_stream_sync(c->stream);
    return finish(rc, name, &o);
}

Error_t spike_dsolve_device(spike_context_t c, integer_t n, integer_t nnz, integer_t nrhs, const integer_t *d_colind,
                            const integer_t *d_rowptr, const double *d_aij, double *d_x, const double *d_b)
{
    return device_solve(c, 0, "spike_dsolve_device", n, nnz, nrhs, d_colind, d_rowptr, d_aij, d_x, d_b);
}
Error_t spike_zsolve_device(spike_context_t c, integer_t n, integer_t nnz, integer_t nrhs, const integer_t *d_colind,
                            const integer_t *d_rowptr, const complex16 *d_aij, complex16 *d_x, const complex16 *d_b)
{
    return device_solve(c, 1, "spike_zsolve_device", n, nnz, nrhs, d_colind, d_rowptr, d_aij, d_x, d_b);
}

/* ------------------------------------------------------------------ */
/* factor handles                                                       */
/* ------------------------------------------------------------------ */
static Error_t factor_common(spike_context_t c, int cplx, const char *name, integer_t n, integer_t nnz,
                             const integer_t *ci, const integer_t *rp, const void *aij, int host, spike_factor_t *out)
{
    if (!out) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: NULL output", name);
    *out = NULL;
    if (n <= 0 || nnz < 0) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: n must be > 0 and nnz >= 0", name);
    if (!ci || !rp || !aij) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: NULL array", name);
    c = spk_get_ctx(c);
    if (!c) return SPIKE_ERROR;
    spike_factor_t f = (spike_factor_t)calloc(1, sizeof *f);
    if (!f) return spk_fail(SPIKE_ERR_MEMORY, "%s: host allocation failed", name);
    f->ctx = c;
    spk_ctx_ref(c);
    f->astream = spk_ctx_astream(c);
    f->is_complex = cplx;
    f->n = n;
    f->nnz = nnz;
    const size_t hs = (cplx ? 2 : 1) * 8;
    int rc = SPK_OK;
    refine_opts o;
    opts_from(c, &o);
    if (host) {
        f->owns = 1;
        rc = spk_malloc_on(&f->o_rowptr, sizeof(int) * ((size_t)n + 1), f->astream);
        if (rc == SPK_OK) rc = spk_malloc_on(&f->o_colind, sizeof(int) * (size_t)(nnz ? nnz : 1), f->astream);
        if (rc == SPK_OK) rc = spk_malloc_on(&f->o_aij, hs * (size_t)(nnz ? nnz : 1), f->astream);
        if (rc == SPK_OK) rc = spk_memcpy_h2d(f->o_rowptr, rp, sizeof(int) * ((size_t)n + 1), c->stream);
        if (rc == SPK_OK && nnz) rc = spk_memcpy_h2d(f->o_colind, ci, sizeof(int) * (size_t)nnz, c->stream);
        if (rc == SPK_OK && nnz) rc = spk_memcpy_h2d(f->o_aij, aij, hs * (size_t)nnz, c->stream);
        f->d_rowptr = (const int *)f->o_rowptr;
        f->d_colind = (const int *)f->o_colind;
        f->d_aij = f->o_aij;
    } else {
        f->d_rowptr = rp;
        f->d_colind = ci;
        f->d_aij = aij;
    }
    int info[3];
    long long l0 = 0;
    if (rc == SPK_OK) rc = spk_analyze(n, nnz, f->d_rowptr, f->d_colind, c->d_scratch, info, c->stream, &l0);
    if (rc == SPK_OK && info[2]) rc = SPK_ECSR;
    if (rc == SPK_OK)
        rc = plan_create(n, nnz, info[0], info[1], cplx, c->mode, c->partitions, RHS_CHUNK, c->stream, c->stream_alloc,
                         &f->plan);
    if (rc == SPK_OK) {
        f->plan->launches = l0;
        f->plan->twist = f->plan->twist_cap && c->twist;
        f->plan->red_fp64 = c->red_fp64 && f->plan->KB <= 64;
        rc = factor_phase(f->plan, f->d_rowptr, f->d_colind, f->d_aij, c->stream);
    }
    if (rc != SPK_OK) {
        spk_stream_sync(c->stream);
        spike_factor_release(f);
        return finish(rc, name, &o);
    }
    *out = f;
    return spk_succeed();
}

Error_t spike_dfactor(spike_context_t c, integer_t n, integer_t nnz, const integer_t *colind, const integer_t *rowptr,
                      const double *aij, spike_factor_t *f)
{
    return factor_common(c, 0, "spike_dfactor", n, nnz, colind, rowptr, aij, 1, f);
}
Error_t spike_zfactor(spike_context_t c, integer_t n, integer_t nnz, const integer_t *colind, const integer_t *rowptr,
                      const complex16 *aij, spike_factor_t *f)
{
    return factor_common(c, 1, "spike_zfactor", n, nnz, colind, rowptr, aij, 1, f);
}
Error_t spike_dfactor_device(spike_context_t c, integer_t n, integer_t nnz, const integer_t *d_colind,
                             const integer_t *d_rowptr, const double *d_aij, spike_factor_t *f)
{
    return factor_common(c, 0, "spike_dfactor_device", n, nnz, d_colind, d_rowptr, d_aij, 0, f);
}

static Error_t solve_factored(spike_factor_t f, int cplx, const char *name, integer_t nrhs, void *x, const void *b,
                              int host)
{
    if (!f || f->released) return spk_fail(SPIKE_ERR_HANDLE, "%s: invalid factor handle", name);
    if (f->is_complex != cplx) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: handle holds another value type", name);
    if (nrhs < 0) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: nrhs must be >= 0", name);
    if (nrhs == 0) return spk_succeed();
    if (!x || !b) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: NULL array", name);
    spike_context_t c = f->ctx;
    spk_plan *P = f->plan;
    const size_t hs = (cplx ? 2 : 1) * 8;
    const size_t nb = (size_t)f->n * nrhs;
    refine_opts o;
    opts_from(c, &o);
    P->launches = 0;
    int rc = ensure(&f->d_r, &f->c_r, hs * (size_t)f->n * P->nrhs_max, f->astream);
    void *dx = x;
    const void *db = b;
    if (host) {
        if (rc == SPK_OK) rc = ensure(&f->d_b, &f->c_b, hs * nb, f->astream);
        if (rc == SPK_OK) rc = ensure(&f->d_x, &f->c_x, hs * nb, f->astream);
        if (rc == SPK_OK) rc = spk_memcpy_h2d(f->d_b, b, hs * nb, c->stream);
        dx = f->d_x;
        db = f->d_b;
    }
    if (rc == SPK_OK) rc = solve_all(P, f->d_rowptr, f->d_colind, f->d_aij, dx, db, f->d_r, nrhs, &o, c->stream);
    if (host && (rc == SPK_OK || rc == SPK_ECONV)) {
        int rc2 = spk_memcpy_d2h(x, f->d_x, hs * nb, c->stream);
        if (rc2 == SPK_OK) rc2 = spk_stream_sync(c->stream);
        if (rc2 != SPK_OK) rc = rc2;
    } else {
        spk_stream_sync(c->stream);
    }
    fill_info(c, P, &o, P->launches);
    return finish(rc, name, &o);
}

Error_t spike_dsolve_factored(spike_factor_t f, integer_t nrhs, double *x, const double *b)
{
    return solve_factored(f, 0, "spike_dsolve_factored", nrhs, x, b, 1);
}
Error_t spike_zsolve_factored(spike_factor_t f, integer_t nrhs, complex16 *x, const complex16 *b)
{
    return solve_factored(f, 1, "spike_zsolve_factored", nrhs, x, b, 1);
}
Error_t spike_dsolve_factored_device(spike_factor_t f, integer_t nrhs, double *d_x, const double *d_b)
{
    return solve_factored(f, 0, "spike_dsolve_factored_device", nrhs, d_x, d_b, 0);
}

Error_t spike_factor_release(spike_factor_t f)
{
    if (!f || f->released) return spk_fail(SPIKE_ERR_HANDLE, "spike_factor_release: invalid factor handle");
    spk_plan_destroy(f->plan);
    spk_free_on(f->o_rowptr, f->astream);
    spk_free_on(f->o_colind, f->astream);
    spk_free_on(f->o_aij, f->astream);
    spk_free_on(f->d_b, f->astream);
    spk_free_on(f->d_x, f->astream);
    spk_free_on(f->d_r, f->astream);
    if (f->ctx && f->ctx->stream) spk_stream_sync(f->ctx->stream);
    if (f->ctx) spk_ctx_unref(f->ctx);
    f->released = 1;
    free(f);
    return spk_succeed();
}

/* ------------------------------------------------------------------ */
/* solve without device allocation                                      */
/* ------------------------------------------------------------------ */
/* Limits of the fixed workspace's schedule (host arrays live on the stack). */
#define NOALLOC_MAX_PARTS 64
#define NOALLOC_MAX_BLOCKS 16384

typedef struct {
    char *base;
    size_t used, cap;
} carve_t;

/* 256-byte aligned slice of the fixed workspace; NULL once it is exhausted */
static void *carve(carve_t *c, size_t bytes)
{
    const size_t off = (c->used + 255) & ~(size_t)255;
    if (off > c->cap || bytes > c->cap - off) {
        c->used = c->cap + 1;
        return NULL;
    }
    c->used = off + bytes;
    return c->base + off;
}

/*
 * spike_dsolve_device_noalloc: the solve of spike_dsolve_device with every
 * temporary carved from the library's fixed per-device workspace
 * (spike_noalloc.cu).  The schedule is built on the stack; the kernels are the
 * same as the allocating path's, fed with pointers into the workspace.
 */
Error_t spike_dsolve_device_noalloc(integer_t n, integer_t nnz, integer_t nrhs, const integer_t *d_colind,
                                    const integer_t *d_rowptr, const double *d_aij, double *d_x, const double *d_b,
                                    void *cuda_stream)
{
    const char *name = "spike_dsolve_device_noalloc";
    if (n < 0 || nnz < 0 || nrhs < 0) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: n, nnz and nrhs must be >= 0", name);
    if (n == 0 || nrhs == 0) return spk_succeed();
    if (!d_colind || !d_rowptr || !d_aij || !d_x || !d_b) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: NULL array", name);
    if (spk_device_count() <= 0) return spk_fail(SPIKE_ERR_NO_DEVICE, "%s: no CUDA device is visible", name);
    void *ws = NULL;
    size_t ws_bytes = 0;
    if (spk_noalloc_scratch(&ws, &ws_bytes) != SPK_OK)
        return spk_fail(SPIKE_ERR_CUDA, "%s: cannot resolve the fixed workspace on this device", name);
    void *stream = cuda_stream;
    carve_t cv = {(char *)ws, 0, ws_bytes};

    /* analysis: bandwidth and CSR checks */
    int info[3];
    long long launches = 0;
    int *d_an = (int *)carve(&cv, 4 * sizeof(int));
    int rc = spk_analyze(n, nnz, d_rowptr, d_colind, d_an, info, stream, &launches);
    if (rc != SPK_OK) return spk_fail_code(rc, name);
    if (info[2]) return spk_fail(SPIKE_ERR_CSR, "%s: invalid CSR (row pointers, column range or ordering)", name);

    /* schedule, as plan_create does, with stack arrays */
    spk_plan P;
    memset(&P, 0, sizeof P);
    const int k = info[0] > info[1] ? info[0] : info[1];
    const int KB = spk_choose_block(k < 1 ? 1 : k);
    if (!KB || spk_factor_smem(KB, 0, SPK_MIXED) == 0)
        return spk_fail(SPIKE_ERR_BANDWIDTH, "%s: bandwidth %d above the supported tile size", name, k);
    int p = choose_partitions(n, KB, 0);
    if (p > NOALLOC_MAX_PARTS) p = NOALLOC_MAX_PARTS;
    int part_start[NOALLOC_MAX_PARTS + 1], blk_off[NOALLOC_MAX_PARTS + 1];
    int cr_count[32];
    long long cr_off[33], cr_moff[33];
    const int nreg = n / p, rem = n % p; /* balanced, as plan_create for an automatic count */
    for (int i = 0; i < p; i++) part_start[i] = i * nreg + (i < rem ? i : rem);
    part_start[p] = n;
    blk_off[0] = 0;
    for (int i = 0; i < p; i++) blk_off[i + 1] = blk_off[i] + (part_start[i + 1] - part_start[i] + KB - 1) / KB;
    if (blk_off[p] > NOALLOC_MAX_BLOCKS)
        return spk_fail(SPIKE_ERR_MEMORY, "%s: %d row blocks exceed the fixed schedule's %d (system too large for the "
                    "%u-byte no-allocation workspace)", name, blk_off[p], NOALLOC_MAX_BLOCKS, SPK_NOALLOC_SCRATCH_BYTES);
    /* the block -> partition map (64 KB): per thread, not on the caller's stack */
    static _Thread_local int blk_part[NOALLOC_MAX_BLOCKS];
    for (int i = 0; i < p; i++)
        for (int b = blk_off[i]; b < blk_off[i + 1]; b++) blk_part[b] = i;
    P.n = n;
    P.nnz = nnz;
    P.ku = info[0];
    P.kl = info[1];
    P.KB = KB;
    P.p = p;
    P.n_iface = p - 1;
    P.is_complex = 0;
    P.mode = SPK_MIXED;
    P.nrhs_max = nrhs < RHS_CHUNK ? nrhs : RHS_CHUNK;
    P.part_start = part_start;
    P.blk_off = blk_off;
    P.total_blocks = blk_off[p];
    P.NP = (long long)P.total_blocks * KB;
    int levels = 0;
    for (int c = P.n_iface; c > 1; c = (c + 1) / 2) levels++;
    P.cr_levels = levels;
    long long tiles = 0, mtiles = 0;
    int c = P.n_iface > 0 ? P.n_iface : 1;
    for (int l = 0; l <= levels; l++) {
        cr_count[l] = c;
        cr_off[l] = tiles;
        cr_moff[l] = mtiles;
        tiles += c;
        mtiles += (l < levels) ? c / 2 : 1;
        c = (c + 1) / 2;
    }
    cr_off[levels + 1] = tiles;
    cr_moff[levels + 1] = mtiles;
    P.cr_count = cr_count;
    P.cr_off = cr_off;
    P.cr_moff = cr_moff;
    P.crg_stride = tiles * 2 * KB;

    /* carve the workspace */
    const size_t fs = 4, hs = 8, TS = (size_t)KB * KB;
    const size_t nif = P.n_iface > 0 ? (size_t)P.n_iface : 1;
    const int nr = P.nrhs_max;
#define CV(ptr, bytes) ptr = carve(&cv, (bytes))
    CV(P.d_part_start, sizeof(int) * (p + 1));
    CV(P.d_blk_off, sizeof(int) * (p + 1));
    CV(P.d_blk_part, sizeof(int) * P.total_blocks);
    CV(P.d_L, fs * TS * P.total_blocks);
    CV(P.d_G, fs * TS * P.total_blocks);
    CV(P.d_E, fs * TS * P.total_blocks);
    CV(P.d_W, fs * TS * P.total_blocks);
    CV(P.d_V, fs * TS * P.total_blocks);
    CV(P.d_Bhat, fs * TS * p);
    CV(P.d_T, fs * TS * 3 * P.total_blocks);
    CV(P.d_RP, hs * TS * nif);
    CV(P.d_RQ, hs * TS * nif);
    CV(P.d_RX, hs * TS * nif);
    CV(P.d_RY, hs * TS * nif);
    CV(P.d_crP, fs * TS * tiles);
    CV(P.d_crQ, fs * TS * tiles);
    CV(P.d_crX, fs * TS * tiles);
    CV(P.d_crY, fs * TS * tiles);
    CV(P.d_crM, fs * TS * 4 * (mtiles > 0 ? mtiles : 1));
    CV(P.d_crg, fs * 2 * (size_t)P.crg_stride * nr);
    CV(P.d_z, fs * (size_t)P.NP * nr);
    CV(P.d_y, fs * (size_t)P.NP * nr);
    CV(P.d_g, hs * nif * 2 * KB * nr);
    CV(P.d_u, hs * nif * 2 * KB * nr);
    CV(P.d_rr, hs * nif * 2 * KB * nr);
    CV(P.d_du, hs * nif * 2 * KB * nr);
    CV(P.d_err, sizeof(unsigned) * 4);
    CV(P.d_norms, sizeof(double) * 2 * nr);
    void *d_r = carve(&cv, hs * (size_t)n * nr);
#undef CV
    if (cv.used > cv.cap)
        return spk_fail(SPIKE_ERR_MEMORY, "%s: the system needs more than the %u-byte no-allocation workspace "
                    "(use spike_dsolve_device)", name, SPK_NOALLOC_SCRATCH_BYTES);
    P.bytes = cv.used;

    rc = spk_memcpy_h2d(P.d_part_start, part_start, sizeof(int) * (p + 1), stream);
    if (rc == SPK_OK) rc = spk_memcpy_h2d(P.d_blk_off, blk_off, sizeof(int) * (p + 1), stream);
    if (rc == SPK_OK) rc = spk_memcpy_h2d(P.d_blk_part, blk_part, sizeof(int) * P.total_blocks, stream);
    P.launches = launches;
    refine_opts o;
    o.max_refine = 3;
    o.red_refine = 0;
    o.tol = 1e-12;
    o.relres_max = 0;
    o.sweeps = 0;
    if (rc == SPK_OK) rc = factor_phase(&P, d_rowptr, d_colind, d_aij, stream);
    if (rc == SPK_OK) rc = solve_all(&P, d_rowptr, d_colind, d_aij, d_x, d_b, d_r, nrhs, &o, stream);
    if (rc != SPK_ECONV) {
        const int rs = spk_stream_sync(stream);
        if (rc == SPK_OK) rc = rs;
    }
    return finish(rc, name, &o);
}
