/*
 * spike_serve.c -- a request loop with continuous batching.
 *
 * No counterpart in the reference (one blocking dspike_core_host call at a
 * time, OpenMP/spike_interfaces.c:43-419).  A server owns `slots` worker
 * threads, each with its own context and CUDA stream; its workspace is
 * allocated stream-ordered, so slots never synchronise the device.
 *
 *   submit   -> the request joins a FIFO; one larger than the whole budget
 *               is rejected on the spot
 *   admit    -> a free slot takes the oldest request once its HBM footprint
 *               (plan + staging, estimated from n, nnz, bandwidth, nrhs) fits
 *               in what running requests leave of the budget; requests that
 *               arrive while others run are admitted as slots and memory free
 *               up, and their GPU work overlaps on the slots' streams
 *   run      -> a request with a factor key whose factorization is resident
 *               solves with it (fresh right-hand side only); a keyed miss
 *               factors into a new resident entry; others take the slot's
 *               own context
 *   complete -> arrival, admission and completion times, relative residual
 *               and refinement sweeps are kept per ticket; p50 / p99 latency
 *               and throughput come from spike_server_stats.
 *
 * Resident factors live in an LRU cache with its own byte budget; an entry in
 * use is never evicted, and a request for a busy entry waits for it.
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "spike_host_internal.h"

typedef struct {
    spike_request_t req;
    long long ticket;
    double t_arrival, t_admit, t_done;
    size_t footprint;
    int state; /* 0 queued, 1 running, 2 done */
    int err;
    char msg[160];
    double relres;
    int sweeps, hit;
} sreq;

typedef struct {
    long long key;
    spike_context_t ctx;
    spike_factor_t f;
    size_t bytes;
    int busy, ready, n;
    double last;
} fentry;

struct spike_server_s {
    spike_server_config_t cfg;
    int device;
    pthread_mutex_t mu;
    pthread_cond_t cv;
    pthread_t *threads;
    int nthreads, stop;
    sreq **reqs;
    long long nreq, cap, next;
    size_t used; /* footprints of running requests */
    fentry *cache;
    int ncache, capcache;
    size_t cache_used;
    struct timespec t0;
    long long completed, rejected, failed, hits, misses;
    long long nqueued, rejected_busy; /* requests waiting for a slot; turned away on a full queue */
    int running, peak_running;
};

static double now_s(const struct spike_server_s *S)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)(t.tv_sec - S->t0.tv_sec) + 1e-9 * (double)(t.tv_nsec - S->t0.tv_nsec);
}

double spike_server_clock(spike_server_t S) { return S ? now_s(S) : 0.0; }

static int host_bandwidth(int n, const int *rp, const int *ci)
{
    int k = 0;
    for (int r = 0; r < n; r++)
        for (int t = rp[r]; t < rp[r + 1]; t++) {
            const int d = ci[t] > r ? ci[t] - r : r - ci[t];
            if (d > k) k = d;
        }
    return k;
}

/* ------------------------------------------------------------------ */
/* factor cache (server lock held)                                      */
/* ------------------------------------------------------------------ */
static fentry *cache_find(struct spike_server_s *S, long long key)
{
    for (int i = 0; i < S->ncache; i++)
        if (S->cache[i].key == key) return &S->cache[i];
    return NULL;
}

static void cache_drop(struct spike_server_s *S, int i)
{
    fentry *e = &S->cache[i];
    if (e->f) spike_factor_release(e->f);
    if (e->ctx) spike_context_destroy(e->ctx);
    S->cache_used -= e->bytes;
    S->cache[i] = S->cache[--S->ncache];
}

/* evict idle least-recently-used entries until `need` more bytes fit */
static void cache_make_room(struct spike_server_s *S, size_t need)
{
    while (S->cache_used + need > S->cfg.cache_budget) {
        int victim = -1;
        for (int i = 0; i < S->ncache; i++)
            if (!S->cache[i].busy && S->cache[i].ready && (victim < 0 || S->cache[i].last < S->cache[victim].last))
                victim = i;
        if (victim < 0) return;
        cache_drop(S, victim);
    }
}

/* ------------------------------------------------------------------ */
/* workers                                                              */
/* ------------------------------------------------------------------ */
static spike_context_t new_context(const struct spike_server_s *S)
{
    spike_context_t c = NULL;
    if (spike_context_create(&c) != SPIKE_SUCCESS) return NULL;
    spike_set_option(c, SPIKE_OPT_PRECISION, S->cfg.precision);
    spike_set_option(c, SPIKE_OPT_TOLERANCE, S->cfg.tolerance);
    spike_set_option(c, SPIKE_OPT_MAX_REFINE, S->cfg.max_refine);
    spike_set_option(c, SPIKE_OPT_STREAM_ALLOC, 1);
    return c;
}

static void run_keyed(struct spike_server_s *S, sreq *q)
{
    const spike_request_t *r = &q->req;
    pthread_mutex_lock(&S->mu);
    fentry *e;
    for (;;) {
        e = cache_find(S, r->factor_key);
        if (!e || (e->ready && !e->busy)) break;
        pthread_cond_wait(&S->cv, &S->mu); /* another slot is creating or using it */
    }
    int hit = e != NULL && e->n == r->n;
    if (e && !hit) { /* same key, another matrix: replace it */
        cache_drop(S, (int)(e - S->cache));
        e = NULL;
    }
    if (!e) {
        if (S->ncache == S->capcache) {
            const int nc = S->capcache ? 2 * S->capcache : 64;
            fentry *ncache = (fentry *)realloc(S->cache, sizeof(fentry) * nc);
            if (!ncache) {
                pthread_mutex_unlock(&S->mu);
                q->err = SPIKE_ERR_MEMORY;
                snprintf(q->msg, sizeof q->msg, "server: host allocation failed");
                return;
            }
            S->cache = ncache;
            S->capcache = nc;
        }
        e = &S->cache[S->ncache++];
        memset(e, 0, sizeof *e);
        e->key = r->factor_key;
        e->n = r->n;
    }
    e->busy = 1;
    const long long key = e->key;
    spike_context_t c = hit ? e->ctx : NULL; /* read under the lock: the cache array may move */
    spike_factor_t f = hit ? e->f : NULL;
    if (hit)
        S->hits++;
    else
        S->misses++;
    pthread_mutex_unlock(&S->mu);

    if (!hit) c = new_context(S);
    Error_t rc = c ? SPIKE_SUCCESS : SPIKE_ERROR;
    if (rc == SPIKE_SUCCESS && !hit) rc = spike_dfactor(c, r->n, r->nnz, r->colind, r->rowptr, r->aij, &f);
    if (rc == SPIKE_SUCCESS) rc = spike_dsolve_factored(f, r->nrhs, r->x, r->b);
    spike_info_t info;
    memset(&info, 0, sizeof info);
    if (c) spike_get_info(c, &info);
    q->hit = hit;
    q->relres = info.relres_max;
    q->sweeps = info.refine_sweeps;
    if (rc != SPIKE_SUCCESS) {
        q->err = spike_last_error_code();
        snprintf(q->msg, sizeof q->msg, "%s", spike_last_error());
    }

    pthread_mutex_lock(&S->mu);
    e = cache_find(S, key); /* the array may have moved */
    if (!hit) {
        if (rc == SPIKE_SUCCESS || f) {
            e->ctx = c;
            e->f = f;
            e->bytes = info.device_bytes + (size_t)r->nnz * 12 + (size_t)(r->n + 1) * 4;
            e->ready = 1;
            S->cache_used += e->bytes;
        } else {
            if (c) spike_context_destroy(c);
            e->ready = 1;
            e->busy = 0;
            cache_drop(S, (int)(e - S->cache));
            e = NULL;
        }
    }
    if (e) {
        e->busy = 0;
        e->last = now_s(S);
        cache_make_room(S, 0);
    }
    pthread_cond_broadcast(&S->cv);
    pthread_mutex_unlock(&S->mu);
}

static void run_fresh(spike_context_t c, sreq *q)
{
    const spike_request_t *r = &q->req;
    Error_t rc = spk_host_solve_ctx(c, SPK_D, "spike_server", r->n, r->nnz, r->nrhs, r->colind, r->rowptr, r->aij,
                                    r->x, r->b);
    spike_info_t info;
    spike_get_info(c, &info);
    q->relres = info.relres_max;
    q->sweeps = info.refine_sweeps;
    if (rc != SPIKE_SUCCESS) {
        q->err = spike_last_error_code();
        snprintf(q->msg, sizeof q->msg, "%s", spike_last_error());
    }
}

static void *worker_main(void *arg)
{
    struct spike_server_s *S = (struct spike_server_s *)arg;
    spk_set_device(S->device);
    spike_context_t c = new_context(S);
    pthread_mutex_lock(&S->mu);
    for (;;) {
        sreq *q = NULL;
        for (;;) {
            while (S->next < S->nreq && S->reqs[S->next]->state == 2) S->next++; /* rejected on submit */
            if (S->next < S->nreq && S->used + S->reqs[S->next]->footprint <= S->cfg.hbm_budget) {
                q = S->reqs[S->next++];
                break;
            }
            if (S->stop) break;
            pthread_cond_wait(&S->cv, &S->mu);
        }
        if (!q) break;
        q->state = 1;
        S->nqueued--;
        q->t_admit = now_s(S);
        S->used += q->footprint;
        if (++S->running > S->peak_running) S->peak_running = S->running;
        pthread_mutex_unlock(&S->mu);

        if (!c) {
            q->err = SPIKE_ERR_CUDA;
            snprintf(q->msg, sizeof q->msg, "server: no context on this slot");
        } else if (q->req.factor_key >= 0) {
            run_keyed(S, q);
        } else {
            run_fresh(c, q);
        }

        pthread_mutex_lock(&S->mu);
        S->used -= q->footprint;
        S->running--;
        q->t_done = now_s(S);
        q->state = 2;
        if (q->err)
            S->failed++;
        else
            S->completed++;
        pthread_cond_broadcast(&S->cv);
    }
    pthread_mutex_unlock(&S->mu);
    if (c) spike_context_destroy(c);
    return NULL;
}

/* ------------------------------------------------------------------ */
/* public API                                                           */
/* ------------------------------------------------------------------ */
Error_t spike_server_create(const spike_server_config_t *cfg, spike_server_t *out)
{
    if (!out || !cfg) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_create: NULL argument");
    *out = NULL;
    if (cfg->slots < 1 || cfg->slots > 64) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_create: slots in [1, 64]");
    if (spk_device_count() <= 0) return spk_fail(SPIKE_ERR_NO_DEVICE, "no CUDA device is visible");
    struct spike_server_s *S = (struct spike_server_s *)calloc(1, sizeof *S);
    if (!S) return spk_fail(SPIKE_ERR_MEMORY, "spike_server_create: host allocation failed");
    S->cfg = *cfg;
    if (S->cfg.tolerance <= 0) S->cfg.tolerance = 1e-12;
    if (S->cfg.max_refine <= 0) S->cfg.max_refine = 3;
    S->device = spk_current_device();
    size_t free_b = 0, total_b = 0;
    spk_mem_info(&free_b, &total_b);
    if (!S->cfg.hbm_budget) S->cfg.hbm_budget = free_b / 10 * 6;
    if (!S->cfg.cache_budget) S->cfg.cache_budget = free_b / 10 * 2;
    clock_gettime(CLOCK_MONOTONIC, &S->t0);
    pthread_mutex_init(&S->mu, NULL);
    pthread_cond_init(&S->cv, NULL);
    S->threads = (pthread_t *)calloc(cfg->slots, sizeof(pthread_t));
    if (!S->threads) {
        free(S);
        return spk_fail(SPIKE_ERR_MEMORY, "spike_server_create: host allocation failed");
    }
    for (int i = 0; i < cfg->slots; i++) {
        if (pthread_create(&S->threads[i], NULL, worker_main, S) != 0) break;
        S->nthreads++;
    }
    if (S->nthreads == 0) {
        free(S->threads);
        free(S);
        return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_create: could not start worker threads");
    }
    *out = S;
    return spk_succeed();
}

Error_t spike_server_submit(spike_server_t S, const spike_request_t *r, long long *ticket)
{
    if (!S || !r || !ticket) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_submit: NULL argument");
    if (r->n < 1 || r->nnz < 0 || r->nrhs < 1 || !r->colind || !r->rowptr || !r->aij || !r->x || !r->b)
        return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_submit: need n >= 1, nrhs >= 1 and host arrays");
    sreq *q = (sreq *)calloc(1, sizeof *q);
    if (!q) return spk_fail(SPIKE_ERR_MEMORY, "spike_server_submit: host allocation failed");
    q->req = *r;
    const int k = r->bandwidth >= 0 ? r->bandwidth : host_bandwidth(r->n, r->rowptr, r->colind);
    q->footprint = spk_solve_footprint(r->n, r->nnz, k, r->nrhs, 0, S->cfg.precision ? SPK_PLAIN : SPK_MIXED, 0);
    pthread_mutex_lock(&S->mu);
    q->t_arrival = r->arrival >= 0 ? r->arrival : now_s(S);
    if (S->nreq == S->cap) {
        const long long nc = S->cap ? 2 * S->cap : 1024;
        sreq **nr = (sreq **)realloc(S->reqs, sizeof(sreq *) * nc);
        if (!nr) {
            pthread_mutex_unlock(&S->mu);
            free(q);
            return spk_fail(SPIKE_ERR_MEMORY, "spike_server_submit: host allocation failed");
        }
        S->reqs = nr;
        S->cap = nc;
    }
    q->ticket = S->nreq;
    S->reqs[S->nreq++] = q;
    if (q->footprint == 0 || q->footprint > S->cfg.hbm_budget) {
        q->state = 2;
        q->t_admit = q->t_done = now_s(S);
        q->err = q->footprint == 0 ? SPIKE_ERR_BANDWIDTH : SPIKE_ERR_MEMORY;
        snprintf(q->msg, sizeof q->msg, q->footprint == 0 ? "bandwidth %d above the largest tile"
                                                          : "footprint above the server's device budget", k);
        S->rejected++;
    } else if (S->cfg.max_queue > 0 && S->nqueued >= S->cfg.max_queue) {
        /* load shedding: a full queue turns the request away at once */
        q->state = 2;
        q->t_admit = q->t_done = now_s(S);
        q->err = SPIKE_ERR_BUSY;
        snprintf(q->msg, sizeof q->msg, "admission queue full (%d waiting)", S->cfg.max_queue);
        S->rejected++;
        S->rejected_busy++;
    } else {
        S->nqueued++;
    }
    *ticket = q->ticket;
    pthread_cond_broadcast(&S->cv);
    pthread_mutex_unlock(&S->mu);
    return spk_succeed();
}

static void fill_status(const sreq *q, spike_request_status_t *st)
{
    st->done = q->state == 2;
    st->error_code = q->err;
    st->relres = q->relres;
    st->sweeps = q->sweeps;
    st->factor_hit = q->hit;
    st->t_arrival = q->t_arrival;
    st->t_admit = q->t_admit;
    st->t_done = q->t_done;
    st->footprint = q->footprint;
}

Error_t spike_server_wait(spike_server_t S, long long ticket, spike_request_status_t *st)
{
    if (!S || !st || ticket < 0) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_wait: bad argument");
    pthread_mutex_lock(&S->mu);
    if (ticket >= S->nreq) {
        pthread_mutex_unlock(&S->mu);
        return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_wait: unknown ticket");
    }
    sreq *q = S->reqs[ticket];
    while (q->state != 2) pthread_cond_wait(&S->cv, &S->mu);
    fill_status(q, st);
    char msg[160];
    snprintf(msg, sizeof msg, "%s", q->msg);
    pthread_mutex_unlock(&S->mu);
    if (st->error_code) return spk_fail(st->error_code, "request %lld: %s", ticket, msg);
    return spk_succeed();
}

Error_t spike_server_poll(spike_server_t S, long long ticket, spike_request_status_t *st)
{
    if (!S || !st || ticket < 0) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_poll: bad argument");
    pthread_mutex_lock(&S->mu);
    if (ticket >= S->nreq) {
        pthread_mutex_unlock(&S->mu);
        return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_poll: unknown ticket");
    }
    fill_status(S->reqs[ticket], st);
    pthread_mutex_unlock(&S->mu);
    return spk_succeed();
}

Error_t spike_server_drain(spike_server_t S)
{
    if (!S) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_drain: NULL server");
    pthread_mutex_lock(&S->mu);
    for (;;) {
        long long pend = 0;
        for (long long i = S->next > 0 ? S->next - 1 : 0; i < S->nreq; i++) pend += S->reqs[i]->state != 2;
        if (!pend && S->running == 0) break;
        pthread_cond_wait(&S->cv, &S->mu);
    }
    pthread_mutex_unlock(&S->mu);
    return spk_succeed();
}

static int cmp_double(const void *a, const void *b)
{
    const double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : x > y;
}

Error_t spike_server_stats(spike_server_t S, spike_server_stats_t *st)
{
    if (!S || !st) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_stats: NULL argument");
    memset(st, 0, sizeof *st);
    pthread_mutex_lock(&S->mu);
    double *lat = (double *)malloc(sizeof(double) * (S->nreq ? S->nreq : 1));
    long long nl = 0;
    double t_first = 1e300, t_last = 0, wait_sum = 0, relres_max = 0;
    for (long long i = 0; i < S->nreq; i++) {
        const sreq *q = S->reqs[i];
        if (q->t_arrival < t_first) t_first = q->t_arrival;
        if (q->state != 2 || q->err) continue;
        if (lat) lat[nl++] = q->t_done - q->t_arrival;
        wait_sum += q->t_admit - q->t_arrival;
        if (q->t_done > t_last) t_last = q->t_done;
        if (!(q->relres <= relres_max)) relres_max = q->relres;
    }
    st->submitted = S->nreq;
    st->completed = S->completed;
    st->rejected = S->rejected;
    st->rejected_busy = S->rejected_busy;
    st->failed = S->failed;
    st->factor_hits = S->hits;
    st->factor_misses = S->misses;
    st->running = S->running;
    st->peak_running = S->peak_running;
    long long queued = 0;
    for (long long i = S->next; i < S->nreq; i++) queued += S->reqs[i]->state == 0;
    st->queued = queued;
    st->device_bytes_running = S->used;
    st->device_bytes_cached = S->cache_used;
    st->resident_factors = S->ncache;
    pthread_mutex_unlock(&S->mu);
    if (lat && nl) {
        qsort(lat, nl, sizeof(double), cmp_double);
        st->latency_p50 = lat[(nl - 1) / 2];
        st->latency_p99 = lat[(long long)ceil(0.99 * nl) - 1 < 0 ? 0 : (long long)ceil(0.99 * nl) - 1];
        st->latency_max = lat[nl - 1];
        st->mean_queue_wait = wait_sum / nl;
        st->throughput = t_last > t_first ? nl / (t_last - t_first) : 0;
    }
    st->relres_max = relres_max;
    free(lat);
    return spk_succeed();
}

Error_t spike_server_destroy(spike_server_t S)
{
    if (!S) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_server_destroy: NULL server");
    spike_server_drain(S);
    pthread_mutex_lock(&S->mu);
    S->stop = 1;
    pthread_cond_broadcast(&S->cv);
    pthread_mutex_unlock(&S->mu);
    for (int i = 0; i < S->nthreads; i++) pthread_join(S->threads[i], NULL);
    while (S->ncache) cache_drop(S, S->ncache - 1);
    for (long long i = 0; i < S->nreq; i++) free(S->reqs[i]);
    free(S->reqs);
    free(S->cache);
    free(S->threads);
    pthread_mutex_destroy(&S->mu);
    pthread_cond_destroy(&S->cv);
    free(S);
    return spk_succeed();
}
