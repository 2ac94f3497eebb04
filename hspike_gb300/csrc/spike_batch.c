/*
 * spike_batch.c -- thousands of independent banded systems in one graph launch.
 *
 * The reference solves one system per call (dspike_core_host,
 * OpenMP/spike_interfaces.c:43-419).  A batch here:
 *
 *   1. reads every system's pattern once (bandwidth, CSR validity);
 *   2. groups the systems by (tile size KB, nrhs); a group lays its systems
 *      end to end in one row space and becomes ONE SPIKE plan whose partitions
 *      never straddle two systems.  No coupling crosses a system boundary, so
 *      the spikes there are zero and those interfaces decouple exactly in the
 *      reduced system: the group's kernels solve all its systems at once;
 *   3. picks each group's tile size and rows per partition -- by timing
 *      candidates on the group itself (the autotuner) or by a rule;
 *   4. captures the whole solve -- every group on its own stream, forked from
 *      and joined back to the context's stream -- into one CUDA graph:
 *        r = b, ||b||                      (batch residual, x = 0)
 *        band tiles, block LU, spikes, reduced factor
 *        x = SPIKE(r)
 *        r = b - A x, relres per system     (FP64)
 *        [x += SPIKE(r), r = b - A x, relres] x (refinement sweeps that the
 *                                              warm-up run needed)
 *   5. runs the graph; a group still above the tolerance gets further eager
 *      sweeps up to the context's limit.
 *
 * The kernels read each system's own CSR, b and x through a device table
 * (spk_sysref): nothing is packed or copied per run, so A's values and b may
 * change between runs (the pattern and the pointers may not).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "spike_host_internal.h"

#define RES_ROWS 1024 /* rows per CTA of the batch residual */
#define TUNE_CANDIDATES 10

typedef struct {
    int KB, nrhs, k;     /* tile size, columns, bandwidth class (max ku, kl) */
    int nsys, *members;  /* indices into the batch's systems */
    long long rows, nnz; /* row space and entries */
    int rpp;             /* target rows per partition */
    int p;               /* partitions */
    int graph_sweeps;    /* refinement sweeps inside the graph */
    spk_plan *P;
    spk_sysref *h_sys;
    spk_sysref *d_sys;
    int *d_part_sys;
    int *d_chunks, nchunks;
    void *d_r;
    double *d_norms, *d_relres;
    unsigned long long *d_worst;
    void *stream;
    double worst;
    int sweeps;
} bgroup;

struct spike_batch_s {
    spike_context_t ctx;
    int count, flags;
    spike_dsystem_t *sys;
    int *ku, *kl;
    int ngroups;
    bgroup *g;
    void *stream; /* the graph is captured and replayed here (never the legacy stream) */
    void *graph;
    long long graph_launches;
    int extra_sweeps, max_graph_sweeps;
    double relres_max, tune_ms;
    size_t bytes;
    int ran;
};

/* ------------------------------------------------------------------ */
/* scheduling rules (pure host logic)                                   */
/* ------------------------------------------------------------------ */
integer_t spike_batch_partitions(integer_t n, integer_t KB, integer_t rows_per_partition)
{
    if (n <= 0 || KB <= 0) return 0;
    if (rows_per_partition < 1) rows_per_partition = 1;
    long long pmax = (long long)n / (2LL * KB); /* two tiles per partition at least */
    if (pmax < 1) pmax = 1;
    long long p = ((long long)n + rows_per_partition / 2) / rows_per_partition;
    if (p < 1) p = 1;
    if (p > pmax) p = pmax;
    return (integer_t)p;
}

/* rule used without the autotuner: enough partitions to fill the GPU (as
 * for a single system), bounded to [2 KB, 256 KB] rows each */
static int rule_rpp(long long rows, int KB)
{
    int sms = spk_sm_count();
    if (sms <= 0) sms = 152;
    const long long per_sm = KB >= 32 ? 2 : KB == 16 ? 8 : 16;
    long long rpp = (rows + sms * per_sm - 1) / (sms * per_sm);
    if (rpp < 2LL * KB) rpp = 2LL * KB;
    if (rpp > 256LL * KB) rpp = 256LL * KB;
    return (int)rpp;
}

/* ------------------------------------------------------------------ */
/* tuner cache: (KB class, nrhs, mode, row-space and mean-size octaves)  */
/* ------------------------------------------------------------------ */
typedef struct {
    int kb0, nrhs, mode, lrows, lmean;
    int KB, rpp;
} tune_entry;
static tune_entry g_tune[256];
static int g_ntune = 0;

static int ilog2ll(long long v)
{
    int l = 0;
    while (v > 1) {
        v >>= 1;
        l++;
    }
    return l;
}

static const tune_entry *tune_find(int kb0, int nrhs, int mode, long long rows, int nsys)
{
    const int lr = ilog2ll(rows), lm = ilog2ll(rows / (nsys > 0 ? nsys : 1));
    for (int i = 0; i < g_ntune; i++)
        if (g_tune[i].kb0 == kb0 && g_tune[i].nrhs == nrhs && g_tune[i].mode == mode && g_tune[i].lrows == lr &&
            g_tune[i].lmean == lm)
            return &g_tune[i];
    return NULL;
}

static void tune_store(int kb0, int nrhs, int mode, long long rows, int nsys, int KB, int rpp)
{
    if (g_ntune >= (int)(sizeof g_tune / sizeof g_tune[0])) return;
    tune_entry e = {kb0, nrhs, mode, ilog2ll(rows), ilog2ll(rows / (nsys > 0 ? nsys : 1)), KB, rpp};
    g_tune[g_ntune++] = e;
}

/* ------------------------------------------------------------------ */
/* group plans                                                          */
/* ------------------------------------------------------------------ */
static void group_free_plan(bgroup *G)
{
    spk_plan_destroy(G->P);
    G->P = NULL;
    spk_free(G->d_part_sys);
    G->d_part_sys = NULL;
}

static void group_free(bgroup *G)
{
    group_free_plan(G);
    spk_free(G->d_sys);
    spk_free(G->d_chunks);
    spk_free(G->d_r);
    spk_free(G->d_norms);
    spk_free(G->d_relres);
    spk_free(G->d_worst);
    spk_stream_destroy(G->stream);
    free(G->h_sys);
    free(G->members);
}

/* partitions of every member for tile KB and rpp rows per partition; builds
 * the plan and the partition -> system map */
static int group_build_plan(struct spike_batch_s *B, bgroup *G, int KB, int rpp)
{
    group_free_plan(G);
    long long p = 0;
    for (int j = 0; j < G->nsys; j++) p += spike_batch_partitions(B->sys[G->members[j]].n, KB, rpp);
    if (p > (1 << 30)) return SPK_EARG;
    int *ps = (int *)malloc(sizeof(int) * (p + 1));
    int *psys = (int *)malloc(sizeof(int) * (p > 0 ? p : 1));
    if (!ps || !psys) {
        free(ps);
        free(psys);
        return SPK_EMEM;
    }
    long long q = 0;
    for (int j = 0; j < G->nsys; j++) {
        const int n = B->sys[G->members[j]].n;
        const int pj = spike_batch_partitions(n, KB, rpp);
        const int nreg = n / pj, rem = n % pj; /* the remainder spread one row each over the first partitions */
        for (int i = 0; i < pj; i++, q++) {
            ps[q] = (int)(G->h_sys[j].row0 + (long long)i * nreg + (i < rem ? i : rem));
            psys[q] = j;
        }
    }
    ps[p] = (int)G->rows;
    int ku = 0, kl = 0;
    for (int j = 0; j < G->nsys; j++) {
        if (B->ku[G->members[j]] > ku) ku = B->ku[G->members[j]];
        if (B->kl[G->members[j]] > kl) kl = B->kl[G->members[j]];
    }
    int rc = spk_plan_build((int)G->rows, G->nnz, ku, kl, KB, 0, B->ctx->mode, (int)p, ps, G->nrhs, G->stream, 0,
                            &G->P);
    if (rc == SPK_OK) G->P->twist = G->P->twist_cap && B->ctx->twist;
    if (rc == SPK_OK) G->P->red_fp64 = B->ctx->red_fp64 && G->P->KB <= 64;
    if (rc == SPK_OK) rc = spk_malloc((void **)&G->d_part_sys, sizeof(int) * (size_t)p);
    if (rc == SPK_OK) rc = spk_memcpy_h2d(G->d_part_sys, psys, sizeof(int) * (size_t)p, G->stream);
    if (rc == SPK_OK) rc = spk_stream_sync(G->stream);
    free(ps);
    free(psys);
    if (rc != SPK_OK) {
        group_free_plan(G);
        return rc;
    }
    G->P->d_sys = G->d_sys;
    G->P->d_part_sys = G->d_part_sys;
    G->KB = KB;
    G->rpp = rpp;
    G->p = (int)p;
    return SPK_OK;
}

/* ------------------------------------------------------------------ */
/* the group's pipeline (eager, or recorded into the graph)             */
/* ------------------------------------------------------------------ */
static int red_iters(const spk_plan *P, const struct spike_batch_s *B)
{
    return B->ctx->red_refine > 0 ? B->ctx->red_refine : (P->mode == SPK_MIXED ? 2 : 1);
}

static int enqueue_residual(bgroup *G, int have_x)
{
    spk_plan *P = G->P;
    TRY(spk_memset(G->d_norms, 0, sizeof(double) * 2 * G->nrhs * (size_t)G->nsys, G->stream));
    return spk_residual_batch(G->d_sys, G->d_chunks, G->nchunks, RES_ROWS, 2 * G->k + 1, G->rows, G->nrhs, 0,
                              have_x, G->d_r, G->d_norms, G->stream, &P->launches);
}

static int enqueue_apply(struct spike_batch_s *B, bgroup *G, int accumulate)
{
    spk_plan *P = G->P;
    TRY(spk_apply(P, G->d_r, G->nrhs, G->stream));
    TRY(spk_reduced_solve(P, G->nrhs, red_iters(P, B), G->stream));
    return spk_retrieve(P, NULL, G->nrhs, accumulate, G->stream);
}

static int enqueue_check(bgroup *G)
{
    TRY(enqueue_residual(G, 1));
    return spk_batch_relres(G->d_norms, G->nsys, G->nrhs, G->d_relres, G->d_worst, G->stream, &G->P->launches);
}

/* r = b; factor; x = SPIKE(r); check; `sweeps` x (correct; check) */
static int enqueue_solve(struct spike_batch_s *B, bgroup *G, int sweeps)
{
    spk_plan *P = G->P;
    TRY(enqueue_residual(G, 0));
    TRY(spk_memset(P->d_err, 0, sizeof(unsigned) * 4, G->stream));
    TRY(spk_factor(P, NULL, NULL, NULL, G->stream));
    TRY(spk_reduced_factor(P, G->stream));
    TRY(enqueue_apply(B, G, 0));
    TRY(enqueue_check(G));
    for (int s = 0; s < sweeps; s++) {
        TRY(enqueue_apply(B, G, 1));
        TRY(enqueue_check(G));
    }
    return SPK_OK;
}

static int read_worst(bgroup *G, double *worst, unsigned *err)
{
    unsigned long long w = 0;
    unsigned e[4] = {0, 0, 0, 0};
    TRY(spk_memcpy_d2h(&w, G->d_worst, sizeof w, G->stream));
    TRY(spk_memcpy_d2h(e, G->P->d_err, sizeof e, G->stream));
    TRY(spk_stream_sync(G->stream));
    memcpy(worst, &w, sizeof w);
    *err = e[0];
    return SPK_OK;
}

static int dev_error(unsigned e)
{
    if (e & SPK_DEV_ERR_TIMEOUT) return SPK_ETIMEOUT;
    if (e & SPK_DEV_ERR_PIVOT) return SPK_EPIVOT;
    if (e & (SPK_DEV_ERR_BAND | SPK_DEV_ERR_CSR)) return SPK_ECSR;
    return SPK_OK;
}

/* eager solve of one group, refining until the tolerance or the limit;
 * *needed = sweeps used */
static int group_solve_eager(struct spike_batch_s *B, bgroup *G, int *needed, double *worst)
{
    unsigned e = 0;
    TRY(enqueue_solve(B, G, 0));
    TRY(read_worst(G, worst, &e));
    TRY(dev_error(e));
    int s = 0;
    while (!(*worst <= B->ctx->tol) && s < B->ctx->max_refine) {
        TRY(enqueue_apply(B, G, 1));
        TRY(enqueue_check(G));
        TRY(read_worst(G, worst, &e));
        s++;
    }
    *needed = s;
    return SPK_OK;
}

/* time one group configuration: a warm-up solve, then the best of two */
static int group_time(struct spike_batch_s *B, bgroup *G, double *ms)
{
    int needed = 0;
    double worst = 0;
    TRY(group_solve_eager(B, G, &needed, &worst));
    G->graph_sweeps = needed;
    double best = 1e30;
    for (int rep = 0; rep < 2; rep++) {
        void *t = NULL;
        double m = 0;
        TRY(spk_timer_begin(&t, G->stream));
        TRY(enqueue_solve(B, G, needed));
        TRY(spk_timer_end(t, G->stream, &m));
        if (m < best) best = m;
    }
    *ms = best;
    return SPK_OK;
}

static int group_tune(struct spike_batch_s *B, bgroup *G, int kb0)
{
    const tune_entry *hit = tune_find(kb0, G->nrhs, B->ctx->mode, G->rows, G->nsys);
    if (hit) return group_build_plan(B, G, hit->KB, hit->rpp);
    int cand_kb[TUNE_CANDIDATES], cand_rpp[TUNE_CANDIDATES], nc = 0;
    const int kbs[2] = {kb0, 2 * kb0};
    for (int a = 0; a < 2; a++) {
        const int KB = kbs[a];
        if (KB > 64 || spk_factor_smem(KB, 0, B->ctx->mode) == 0) continue;
        if (a == 1 && kb0 >= 16) continue; /* larger tiles only pay for the smallest bands */
        const int mult[4] = {16, 32, 64, 128};
        for (int i = 0; i < 4 && nc < TUNE_CANDIDATES; i++) {
            cand_kb[nc] = KB;
            cand_rpp[nc] = KB * mult[i];
            nc++;
        }
    }
    double best = 1e30;
    int bk = kb0, br = rule_rpp(G->rows, kb0);
    for (int c = 0; c < nc; c++) {
        double ms = 0;
        int rc = group_build_plan(B, G, cand_kb[c], cand_rpp[c]);
        if (rc == SPK_OK) rc = group_time(B, G, &ms);
        if (rc == SPK_EMEM) continue; /* candidate does not fit: skip it */
        if (rc != SPK_OK) return rc;
        B->tune_ms += ms * 3;
        if (ms < best) {
            best = ms;
            bk = cand_kb[c];
            br = cand_rpp[c];
        }
    }
    tune_store(kb0, G->nrhs, B->ctx->mode, G->rows, G->nsys, bk, br);
    return group_build_plan(B, G, bk, br);
}

/* ------------------------------------------------------------------ */
/* public API                                                           */
/* ------------------------------------------------------------------ */
static void batch_free(struct spike_batch_s *B)
{
    if (!B) return;
    spk_graph_destroy(B->graph);
    for (int i = 0; i < B->ngroups; i++) group_free(&B->g[i]);
    spk_stream_destroy(B->stream);
    free(B->g);
    free(B->sys);
    free(B->ku);
    free(B->kl);
    if (B->ctx) spk_ctx_unref(B->ctx);
    free(B);
}

static int cmp_group(const void *a, const void *b)
{
    const int *x = (const int *)a, *y = (const int *)b;
    for (int i = 0; i < 3; i++)
        if (x[i] != y[i]) return x[i] < y[i] ? -1 : 1;
    return 0;
}

static int capture(struct spike_batch_s *B)
{
    void *main = B->stream;
    long long l0 = 0;
    for (int i = 0; i < B->ngroups; i++) l0 += B->g[i].P->launches;
    TRY(spk_capture_begin(main));
    int rc = SPK_OK;
    for (int i = 0; i < B->ngroups && rc == SPK_OK; i++) {
        bgroup *G = &B->g[i];
        rc = spk_stream_fork(main, G->stream);
        if (rc == SPK_OK) rc = enqueue_solve(B, G, G->graph_sweeps);
        if (rc == SPK_OK) rc = spk_stream_fork(G->stream, main);
    }
    void *exec = NULL;
    const int rc2 = spk_capture_end(main, &exec);
    if (rc != SPK_OK) {
        spk_graph_destroy(exec);
        return rc;
    }
    TRY(rc2);
    B->graph = exec;
    long long l1 = 0;
    for (int i = 0; i < B->ngroups; i++) l1 += B->g[i].P->launches;
    B->graph_launches = l1 - l0;
    return SPK_OK;
}

Error_t spike_dbatch_create(spike_context_t ctx, integer_t count, const spike_dsystem_t *systems, int flags,
                            spike_batch_t *out)
{
    const char *W = "spike_dbatch_create";
    if (!out) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: NULL output", W);
    *out = NULL;
    if (count < 1 || !systems) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: need count >= 1 and a system array", W);
    for (int i = 0; i < count; i++) {
        const spike_dsystem_t *s = &systems[i];
        if (s->n < 1 || s->nnz < 0 || s->nrhs < 1 || s->nrhs > 32 || !s->d_colind || !s->d_rowptr || !s->d_aij ||
            !s->d_x || !s->d_b)
            return spk_fail(SPIKE_ERR_ARGUMENT, "%s: system %d: need n >= 1, nnz >= 0, 1 <= nrhs <= 32 and device "
                            "arrays", W, i);
    }
    ctx = spk_get_ctx(ctx);
    if (!ctx) return SPIKE_ERROR;
    struct spike_batch_s *B = (struct spike_batch_s *)calloc(1, sizeof *B);
    if (!B) return spk_fail(SPIKE_ERR_MEMORY, "%s: host allocation failed", W);
    B->ctx = ctx;
    spk_ctx_ref(ctx);
    B->count = count;
    B->flags = flags;
    B->sys = (spike_dsystem_t *)malloc(sizeof(spike_dsystem_t) * count);
    B->ku = (int *)malloc(sizeof(int) * count);
    B->kl = (int *)malloc(sizeof(int) * count);
    int *key = (int *)malloc(sizeof(int) * 4 * count); /* KB, nrhs, k, index */
    int rc = (B->sys && B->ku && B->kl && key) ? SPK_OK : SPK_EMEM;
    if (rc == SPK_OK) memcpy(B->sys, systems, sizeof(spike_dsystem_t) * count);
    if (rc == SPK_OK) rc = spk_stream_create(&B->stream);
    /* 1. patterns */
    for (int i = 0; rc == SPK_OK && i < count; i++) {
        int info[3];
        rc = spk_analyze(B->sys[i].n, B->sys[i].nnz, B->sys[i].d_rowptr, B->sys[i].d_colind, ctx->d_scratch, info,
                         ctx->stream, NULL);
        if (rc != SPK_OK) break;
        if (info[2]) {
            free(key);
            batch_free(B);
            return spk_fail(SPIKE_ERR_CSR, "%s: system %d: invalid CSR (row pointers, column range or ordering)", W,
                            i);
        }
        B->ku[i] = info[0];
        B->kl[i] = info[1];
        const int k = info[0] > info[1] ? info[0] : info[1];
        const int KB = spk_choose_block(k < 1 ? 1 : k);
        if (!KB || spk_factor_smem(KB, 0, ctx->mode) == 0) {
            free(key);
            batch_free(B);
            return spk_fail(SPIKE_ERR_BANDWIDTH, "%s: system %d: bandwidth %d above the largest tile of this precision", W, i, k);
        }
        key[4 * i] = KB;
        key[4 * i + 1] = B->sys[i].nrhs;
        key[4 * i + 2] = k;
        key[4 * i + 3] = i;
    }
    if (rc != SPK_OK) {
        free(key);
        batch_free(B);
        return spk_fail_code(rc, W);
    }
    /* 2. groups by (KB, nrhs); a group's row space must fit an int */
    qsort(key, count, 4 * sizeof(int), cmp_group);
    B->g = (bgroup *)calloc(count, sizeof(bgroup));
    if (!B->g) rc = SPK_EMEM;
    for (int i = 0; rc == SPK_OK && i < count;) {
        int j = i;
        long long rows = 0;
        while (j < count && key[4 * j] == key[4 * i] && key[4 * j + 1] == key[4 * i + 1] &&
               rows + B->sys[key[4 * j + 3]].n < (1LL << 30))
            rows += B->sys[key[4 * j + 3]].n, j++;
        bgroup *G = &B->g[B->ngroups++];
        G->KB = key[4 * i];
        G->nrhs = key[4 * i + 1];
        G->nsys = j - i;
        G->members = (int *)malloc(sizeof(int) * G->nsys);
        G->h_sys = (spk_sysref *)calloc(G->nsys, sizeof(spk_sysref));
        if (!G->members || !G->h_sys) {
            rc = SPK_EMEM;
            break;
        }
        long long row0 = 0, nchunks = 0;
        for (int q = 0; q < G->nsys; q++) {
            const int s = key[4 * (i + q) + 3];
            const spike_dsystem_t *S = &B->sys[s];
            G->members[q] = s;
            if (key[4 * (i + q) + 2] > G->k) G->k = key[4 * (i + q) + 2];
            G->h_sys[q].rowptr = S->d_rowptr;
            G->h_sys[q].colind = S->d_colind;
            G->h_sys[q].aij = S->d_aij;
            G->h_sys[q].x = S->d_x;
            G->h_sys[q].b = S->d_b;
            G->h_sys[q].row0 = row0;
            G->h_sys[q].n = S->n;
            row0 += S->n;
            G->nnz += S->nnz;
            nchunks += (S->n + RES_ROWS - 1) / RES_ROWS;
        }
        G->rows = row0;
        G->nchunks = (int)nchunks;
        int *chunks = (int *)malloc(sizeof(int) * 2 * (size_t)nchunks);
        if (!chunks) {
            rc = SPK_EMEM;
            break;
        }
        for (int q = 0, c = 0; q < G->nsys; q++)
            for (int r = 0; r < G->h_sys[q].n; r += RES_ROWS, c++) {
                chunks[2 * c] = q;
                chunks[2 * c + 1] = r;
            }
        rc = spk_stream_create(&G->stream);
#define GA(ptr, bytes)                                                                                          \
    if (rc == SPK_OK) rc = spk_malloc((void **)&(ptr), (bytes))
        GA(G->d_sys, sizeof(spk_sysref) * G->nsys);
        GA(G->d_chunks, sizeof(int) * 2 * (size_t)nchunks);
        GA(G->d_r, sizeof(double) * (size_t)G->rows * G->nrhs);
        GA(G->d_norms, sizeof(double) * 2 * G->nrhs * (size_t)G->nsys);
        GA(G->d_relres, sizeof(double) * G->nsys);
        GA(G->d_worst, sizeof(unsigned long long));
#undef GA
        if (rc == SPK_OK) rc = spk_memcpy_h2d(G->d_sys, G->h_sys, sizeof(spk_sysref) * G->nsys, G->stream);
        if (rc == SPK_OK) rc = spk_memcpy_h2d(G->d_chunks, chunks, sizeof(int) * 2 * (size_t)nchunks, G->stream);
        if (rc == SPK_OK) rc = spk_stream_sync(G->stream);
        free(chunks);
        i = j;
    }
    free(key);
    /* 3. schedules: tuned or by rule; 4. warm-up run (also the sweep count) */
    for (int i = 0; rc == SPK_OK && i < B->ngroups; i++) {
        bgroup *G = &B->g[i];
        if (flags & SPIKE_BATCH_AUTOTUNE)
            rc = group_tune(B, G, G->KB);
        else
            rc = group_build_plan(B, G, G->KB, rule_rpp(G->rows, G->KB));
        if (rc == SPK_OK) rc = group_solve_eager(B, G, &G->graph_sweeps, &G->worst);
        if (rc == SPK_OK && G->graph_sweeps > B->max_graph_sweeps) B->max_graph_sweeps = G->graph_sweeps;
    }
    if (rc == SPK_OK && !(flags & SPIKE_BATCH_NO_GRAPH)) rc = capture(B);
    if (rc != SPK_OK) {
        batch_free(B);
        return spk_fail_code(rc, W);
    }
    for (int i = 0; i < B->ngroups; i++)
        B->bytes += B->g[i].P->bytes + sizeof(double) * (size_t)B->g[i].rows * B->g[i].nrhs;
    *out = B;
    return spk_succeed();
}

Error_t spike_batch_run(spike_batch_t B)
{
    const char *W = "spike_batch_run";
    if (!B) return spk_fail(SPIKE_ERR_HANDLE, "%s: NULL batch", W);
    int rc = SPK_OK;
    if (B->graph) {
        /* after the caller's queued work on the context's stream */
        rc = spk_stream_fork(B->ctx->stream, B->stream);
        if (rc == SPK_OK) rc = spk_graph_launch(B->graph, B->stream);
        if (rc == SPK_OK) rc = spk_stream_sync(B->stream);
        for (int i = 0; rc == SPK_OK && i < B->ngroups; i++) B->g[i].sweeps = B->g[i].graph_sweeps;
    } else {
        for (int i = 0; rc == SPK_OK && i < B->ngroups; i++) {
            rc = spk_stream_fork(B->ctx->stream, B->g[i].stream);
            if (rc == SPK_OK) rc = enqueue_solve(B, &B->g[i], B->g[i].graph_sweeps);
            B->g[i].sweeps = B->g[i].graph_sweeps;
        }
    }
    /* convergence and device errors of every group; eager sweeps where needed */
    B->extra_sweeps = 0;
    B->relres_max = 0;
    int conv = 1;
    for (int i = 0; rc == SPK_OK && i < B->ngroups; i++) {
        bgroup *G = &B->g[i];
        unsigned e = 0;
        rc = read_worst(G, &G->worst, &e);
        if (rc == SPK_OK) rc = dev_error(e);
        while (rc == SPK_OK && !(G->worst <= B->ctx->tol) && G->sweeps < B->ctx->max_refine) {
            rc = enqueue_apply(B, G, 1);
            if (rc == SPK_OK) rc = enqueue_check(G);
            if (rc == SPK_OK) rc = read_worst(G, &G->worst, &e);
            G->sweeps++;
            B->extra_sweeps++;
        }
        if (!(G->worst <= B->relres_max)) B->relres_max = G->worst;
        if (!(G->worst <= B->ctx->tol)) conv = 0;
    }
    /* later work on the context's stream sees x */
    if (rc == SPK_OK && B->graph) rc = spk_stream_fork(B->stream, B->ctx->stream);
    for (int i = 0; rc == SPK_OK && i < B->ngroups; i++) rc = spk_stream_fork(B->g[i].stream, B->ctx->stream);
    if (rc == SPK_OK) rc = spk_stream_sync(B->ctx->stream);
    B->ran = 1;
    if (rc != SPK_OK) return spk_fail_code(rc, W);
    if (!conv)
        return spk_fail(SPIKE_ERR_CONVERGENCE, "%s: relative residual %.3e above tolerance %.3e", W, B->relres_max,
                        B->ctx->tol);
    return spk_succeed();
}

Error_t spike_batch_relres(spike_batch_t B, double *relres)
{
    if (!B || !relres) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_batch_relres: NULL argument");
    for (int i = 0; i < B->ngroups; i++) {
        bgroup *G = &B->g[i];
        double *tmp = (double *)malloc(sizeof(double) * G->nsys);
        if (!tmp) return spk_fail(SPIKE_ERR_MEMORY, "spike_batch_relres: host allocation failed");
        int rc = spk_memcpy_d2h(tmp, G->d_relres, sizeof(double) * G->nsys, G->stream);
        if (rc == SPK_OK) rc = spk_stream_sync(G->stream);
        if (rc != SPK_OK) {
            free(tmp);
            return spk_fail_code(rc, "spike_batch_relres");
        }
        for (int j = 0; j < G->nsys; j++) relres[G->members[j]] = tmp[j];
        free(tmp);
    }
    return spk_succeed();
}

Error_t spike_batch_get_info(spike_batch_t B, spike_batch_info_t *info)
{
    if (!B || !info) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_batch_get_info: NULL argument");
    memset(info, 0, sizeof *info);
    info->systems = B->count;
    info->groups = B->ngroups;
    info->graph_sweeps = B->max_graph_sweeps;
    info->extra_sweeps = B->extra_sweeps;
    info->relres_max = B->relres_max;
    info->graph_kernel_launches = B->graph_launches;
    info->device_bytes = B->bytes;
    info->tune_ms = B->tune_ms;
    info->graph = B->graph != NULL;
    return spk_succeed();
}

Error_t spike_batch_group(spike_batch_t B, integer_t i, spike_batch_group_t *g)
{
    if (!B || !g || i < 0 || i >= B->ngroups) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_batch_group: bad argument");
    const bgroup *G = &B->g[i];
    g->block = G->KB;
    g->nrhs = G->nrhs;
    g->bandwidth = G->k;
    g->systems = G->nsys;
    g->partitions = G->p;
    g->rows_per_partition = G->rpp;
    g->rows = G->rows;
    g->nnz = G->nnz;
    g->graph_sweeps = G->graph_sweeps;
    return spk_succeed();
}

Error_t spike_batch_destroy(spike_batch_t B)
{
    if (!B) return spk_fail(SPIKE_ERR_HANDLE, "spike_batch_destroy: NULL batch");
    spk_stream_sync(B->ctx->stream);
    batch_free(B);
    return spk_succeed();
}
