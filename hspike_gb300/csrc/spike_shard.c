/*
 * spike_shard.c -- one system's SPIKE partitions sharded across ranks.
 *
 * The reference's distributed solve (MPI/spike_dm.c:21-202 with the
 * transfers of MPI/spike_mpi.c:450-674) is a master/worker exchange: the
 * master cuts A into partitions and sends each worker its A_i, f_i and the
 * coupling blocks B_i, C_i; workers factor, solve for their spikes and send
 * the tips back; the master assembles and solves the reduced system and
 * scatters the x tips; workers retrieve their x_i and the master gathers x.
 *
 * Here every rank already holds the CSR rows of its contiguous range of
 * partitions (spike_shard_range) and keeps its x; only the reduced system
 * moves.  Each rank solves a local system on its own GPU with the ordinary
 * single-system kernels: its rows, renumbered, with a band of h = 8 KB
 * identity rows on either side ("halo partitions").  The rows next to a halo
 * keep their couplings to the neighbouring ranks' rows, which in the local
 * numbering fall inside the halos, so the partitions next to the halos get
 * their W (first) and V (last) spikes from the true couplings, exactly as in
 * a single-GPU solve of the whole matrix; the halo partitions themselves have
 * no couplings, so their spikes vanish and their x rows are whatever their
 * right-hand side says.  Then:
 *
 *   factor      local band tiles, chains, spikes and interface blocks;
 *               every rank's interface blocks go to rank 0 (gather), which
 *               assembles the global reduced system -- the halves of a
 *               boundary interface come from the two ranks that own its two
 *               partitions -- and factors it;
 *   per sweep   local right-hand-side sweep -> y tips to rank 0 -> reduced
 *               solve on rank 0 -> each rank's interface unknowns back
 *               (scatter) -> local retrieval; KB rows of x with each
 *               neighbour into the halo rows; local FP64 residual over the
 *               local rows (the halo rows contribute zero: their b is set to
 *               their x) -> norms summed over ranks -> the same stopping
 *               decision on every rank.
 *
 * An error on any rank is made known to all (an error word summed over the
 * ranks after each local phase) so that no rank waits in a collective the
 * others have left.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "spike_host_internal.h"

/* the reference's partition rule: partition i starts at row i floor(n / p) */
static long long part_row(int n, int p, int i) { return i < p ? (long long)i * (n / p) : (long long)n; }

Error_t spike_shard_range(integer_t n, integer_t p, integer_t size, integer_t rank, integer_t *part0, integer_t *part1,
                          integer_t *row0, integer_t *row1)
{
    if (n < 1 || p < 1 || p > n || size < 1 || size > p || rank < 0 || rank >= size || !part0 || !part1 || !row0 ||
        !row1)
        return spk_fail(SPIKE_ERR_ARGUMENT, "spike_shard_range: need 1 <= p <= n, 1 <= size <= p, 0 <= rank < size");
    const int a = (int)((long long)p * rank / size), b = (int)((long long)p * (rank + 1) / size);
    *part0 = a;
    *part1 = b;
    *row0 = (int)part_row(n, p, a);
    *row1 = (int)part_row(n, p, b);
    return spk_succeed();
}

/* records per rank slot: the most local interfaces any rank has */
static int slot_records(int p, int size) { return (p + size - 1) / size + 1; }

Error_t spike_shard_assemble(integer_t p, integer_t size, integer_t left_len, integer_t right_len,
                             const double *slots, double *global)
{
    if (p < 2 || size < 1 || size > p || left_len < 0 || right_len < 0 || !slots || !global)
        return spk_fail(SPIKE_ERR_ARGUMENT, "spike_shard_assemble: bad argument");
    const size_t rec = (size_t)left_len + (size_t)right_len;
    const size_t slot = rec * (size_t)slot_records(p, size);
    for (int r = 0; r < size; r++) {
        const int a = (int)((long long)p * r / size), b = (int)((long long)p * (r + 1) / size);
        const int nloc = b - a + 1; /* local interfaces j = 0 .. b - a */
        for (int j = 0; j < nloc; j++) {
            const int g = a - 1 + j; /* global interface between partitions g and g + 1 */
            if (g < 0 || g > p - 2) continue;
            const double *src = slots + (size_t)r * slot + (size_t)j * rec;
            double *dst = global + (size_t)g * rec;
            /* partition g is this rank's unless j = 0; partition g + 1 unless j = nloc - 1 */
            if (j > 0) memcpy(dst, src, sizeof(double) * (size_t)left_len);
            if (j < nloc - 1) memcpy(dst + left_len, src + left_len, sizeof(double) * (size_t)right_len);
        }
    }
    return spk_succeed();
}

Error_t spike_shard_split(integer_t p, integer_t size, integer_t left_len, integer_t right_len, const double *global,
                          double *slots)
{
    if (p < 2 || size < 1 || size > p || left_len < 0 || right_len < 0 || !slots || !global)
        return spk_fail(SPIKE_ERR_ARGUMENT, "spike_shard_split: bad argument");
    const size_t rec = (size_t)left_len + (size_t)right_len;
    const int nrec = slot_records(p, size);
    const size_t slot = rec * (size_t)nrec;
    for (int r = 0; r < size; r++) {
        const int a = (int)((long long)p * r / size), b = (int)((long long)p * (r + 1) / size);
        for (int j = 0; j < nrec; j++) {
            const int g = a - 1 + j;
            double *dst = slots + (size_t)r * slot + (size_t)j * rec;
            if (j <= b - a && g >= 0 && g <= p - 2)
                memcpy(dst, global + (size_t)g * rec, sizeof(double) * rec);
            else
                memset(dst, 0, sizeof(double) * rec);
        }
    }
    return spk_succeed();
}

/* ------------------------------------------------------------------ */
/* the collective solve                                                */
/* ------------------------------------------------------------------ */

/* The largest halo: 8 tiles of the largest block (128 rows).  The rank's rows
 * sit this many rows (entries) into the local buffers whatever the block size
 * turns out to be, so their copies start before the bandwidth is known; the
 * local CSR begins SHARD_HALO_MAX - h rows (entries) in, h = 8 KB. */
#define SHARD_HALO_MAX (8 * 128)

/* What a sharded solve holds on its rank, kept on the context for the next
 * call of the same shape: the plans and device buffers are most of a call's
 * setup otherwise. */
typedef struct {
    /* the rank's rows: keys of the buffers */
    int n, p, nrhs, rows, size, rank, part0, part1, row0;
    long long nnz;
    int *d_rp_buf, *d_ci_buf; /* rows + 1 + 2 SHARD_HALO_MAX / nnz + 2 SHARD_HALO_MAX */
    double *d_a_buf;          /* nnz + 2 SHARD_HALO_MAX */
    /* the block size and precision: keys of the plans */
    int KB, mode, h, nloc_if, nrec, n_loc;
    long long nnz_loc;
    spk_plan *P;  /* the local system's plan */
    spk_plan *Pg; /* rank 0: the global reduced system */
    double *d_b, *d_x, *d_r;
    /* host staging */
    double *h_loc;   /* this rank's slot */
    double *h_all;   /* rank 0: every rank's slot */
    double *h_glob;  /* rank 0: the global records */
    double *h_dev;   /* device-layout staging (interface blocks or reduced right-hand side) */
    double *h_halo;  /* 4 KB x nrhs: to lo, to hi, from lo, from hi */
    /* this call */
    const spike_comm_t *cm;
    spike_context_t c;
    int *d_rp, *d_ci; /* the local CSR, inside the buffers above */
    double *d_a;
} shard_t;

static void shard_free_plans(shard_t *S)
{
    spk_plan_destroy(S->P);
    spk_plan_destroy(S->Pg);
    spk_free(S->d_b);
    spk_free(S->d_x);
    spk_free(S->d_r);
    spk_host_free(S->h_loc);
    spk_host_free(S->h_all);
    spk_host_free(S->h_glob);
    spk_host_free(S->h_dev);
    spk_host_free(S->h_halo);
    S->P = S->Pg = NULL;
    S->d_b = S->d_x = S->d_r = NULL;
    S->h_loc = S->h_all = S->h_glob = S->h_dev = S->h_halo = NULL;
    S->KB = 0;
}

void spk_shard_release(spike_context_t c)
{
    shard_t *S = c ? (shard_t *)c->shard : NULL;
    if (!S) return;
    spk_stream_sync(c->stream);
    if (c->copy_stream) spk_stream_sync(c->copy_stream);
    shard_free_plans(S);
    spk_free(S->d_rp_buf);
    spk_free(S->d_ci_buf);
    spk_free(S->d_a_buf);
    free(S);
    c->shard = NULL;
}

/* the context's shard state for this shape, its buffers allocated */
static int shard_buffers(spike_context_t c, const spike_comm_t *cm, int n, int p, int nrhs, int rows, long long nnz,
                         int part0, int part1, int row0, shard_t **out)
{
    shard_t *S = (shard_t *)c->shard;
    if (S && (S->n != n || S->p != p || S->nrhs != nrhs || S->rows != rows || S->nnz != nnz || S->size != cm->size ||
              S->rank != cm->rank || S->row0 != row0)) {
        spk_shard_release(c);
        S = NULL;
    }
    if (!S) {
        S = (shard_t *)calloc(1, sizeof *S);
        if (!S) return SPK_EMEM;
        c->shard = S;
        S->n = n;
        S->p = p;
        S->nrhs = nrhs;
        S->rows = rows;
        S->nnz = nnz;
        S->size = cm->size;
        S->rank = cm->rank;
        S->part0 = part0;
        S->part1 = part1;
        S->row0 = row0;
        const size_t H = SHARD_HALO_MAX;
        TRY(spk_malloc((void **)&S->d_rp_buf, sizeof(int) * ((size_t)rows + 1 + 2 * H)));
        TRY(spk_malloc((void **)&S->d_ci_buf, sizeof(int) * ((size_t)nnz + 2 * H)));
        TRY(spk_malloc((void **)&S->d_a_buf, sizeof(double) * ((size_t)nnz + 2 * H)));
    }
    *out = S;
    return SPK_OK;
}

/* the local plan (halo partition, the rank's partitions, halo partition),
 * rank 0's global reduced plan and the staging, for tile size KB */
static int shard_plans(shard_t *S, int KB)
{
    spike_context_t c = S->c;
    if (S->P && S->KB == KB && S->mode == c->mode) return SPK_OK;
    shard_free_plans(S);
    const int h = 8 * KB, m = S->rows, nl = m + 2 * h, nr = S->nrhs, p = S->p;
    S->h = h;
    S->n_loc = nl;
    S->nnz_loc = S->nnz + 2LL * h;
    S->nloc_if = S->part1 - S->part0 + 1;
    S->nrec = slot_records(p, S->size);
    if (S->nnz_loc > 0x7fffffffLL) return SPK_EARG;
    const int np = S->part1 - S->part0, pl = np + 2;
    int *ps = (int *)malloc(sizeof(int) * ((size_t)pl + 1));
    if (!ps) return SPK_EMEM;
    ps[0] = 0;
    for (int j = 0; j <= np; j++) ps[1 + j] = h + (int)(part_row(S->n, p, S->part0 + j) - S->row0);
    ps[pl] = nl;
    int rc = spk_plan_build(nl, S->nnz_loc, KB, KB, KB, 0, c->mode, pl, ps, nr, c->stream, 0, &S->P);
    free(ps);
    TRY(rc);
    const size_t vb = sizeof(double) * (size_t)nl * nr;
    TRY(spk_malloc((void **)&S->d_b, vb));
    TRY(spk_malloc((void **)&S->d_x, vb));
    TRY(spk_malloc((void **)&S->d_r, vb));
    const size_t TS = (size_t)KB * KB, rec_blk = 4 * TS, rec_red = (size_t)2 * KB * nr;
    const size_t rec_max = rec_blk > rec_red ? rec_blk : rec_red;
    /* host staging, page-locked: the records travel between the device and
     * the exchanges through it */
    TRY(spk_host_alloc((void **)&S->h_loc, sizeof(double) * rec_max * S->nrec));
    TRY(spk_host_alloc((void **)&S->h_dev, sizeof(double) * rec_max * (size_t)(p > S->nrec ? p : S->nrec)));
    TRY(spk_host_alloc((void **)&S->h_halo, sizeof(double) * 4 * (size_t)KB * nr));
    if (S->rank == 0) {
        TRY(spk_host_alloc((void **)&S->h_all, sizeof(double) * rec_max * S->nrec * (size_t)S->size));
        TRY(spk_host_alloc((void **)&S->h_glob, sizeof(double) * rec_max * (size_t)p));
        TRY(spk_plan_reduced_build(p, KB, 0, c->mode, nr, &S->Pg));
    }
    S->KB = KB;
    S->mode = c->mode;
    return SPK_OK;
}

static int device_error(spk_plan *P, void *stream)
{
    unsigned e[4] = {0, 0, 0, 0};
    TRY(spk_memcpy_d2h(e, P->d_err, sizeof e, stream));
    TRY(spk_stream_sync(stream));
    if (e[0] & SPK_DEV_ERR_TIMEOUT) return SPK_ETIMEOUT;
    if (e[0] & SPK_DEV_ERR_PIVOT) return SPK_EPIVOT;
    if (e[0] & (SPK_DEV_ERR_BAND | SPK_DEV_ERR_CSR)) return SPK_ECSR;
    return SPK_OK;
}

/* Every rank's status summed over the ranks: SPK_OK when all succeeded, else
 * the first failing rank's code (its own message stays on that rank; the
 * others report that a peer failed). */
static int agree(shard_t *S, int rc, int *peer_failed)
{
    const int size = S->cm->size;
    double *v = (double *)calloc((size_t)size, sizeof(double));
    if (!v) return SPK_EMEM;
    v[S->cm->rank] = (double)rc;
    const int crc = S->cm->allreduce_sum(S->cm->user, v, size);
    int out = SPK_OK;
    for (int r = 0; r < size && out == SPK_OK; r++)
        if (v[r] != 0.0) out = (int)v[r];
    free(v);
    if (crc != 0) return SPK_ECUDA;
    *peer_failed = (out != SPK_OK && rc == SPK_OK);
    return out;
}

/* This rank's rows renumbered with h identity rows on either side, in place
 * in the buffers that received them (the values are already there or on the
 * way, behind an event on the context's stream), and the local right-hand
 * side with zero halo rows. */
static int shard_local(shard_t *S, const double *b)
{
    const int h = S->h, m = S->rows, nl = S->n_loc, nr = S->nrhs;
    const size_t off = (size_t)SHARD_HALO_MAX - (size_t)h;
    S->d_rp = S->d_rp_buf + off;
    S->d_ci = S->d_ci_buf + off;
    S->d_a = S->d_a_buf + off;
    void *st = S->c->stream;
    const size_t vb = sizeof(double) * (size_t)nl * nr;
    TRY(spk_shard_local(m, S->nnz, h, S->row0, S->d_rp, S->d_ci, S->d_a, st));
    TRY(spk_memset(S->d_b, 0, vb, st));
    for (int k = 0; k < nr; k++)
        TRY(spk_memcpy_h2d(S->d_b + (size_t)k * nl + h, b + (size_t)k * m, sizeof(double) * m, st));
    return spk_memset(S->d_x, 0, vb, st);
}

/* Local interface j's record of the interface blocks: P X (bottom tips of its
 * left partition) | Q Y (top tips of its right partition), KB x KB each,
 * copied from the plan's block arrays straight into the records (pitched) */
static int pack_blocks(shard_t *S)
{
    const size_t TS = (size_t)S->KB * S->KB, ni = (size_t)S->nloc_if, rec = 4 * TS;
    spk_plan *P = S->P;
    const void *src[4] = {P->d_RP, P->d_RX, P->d_RQ, P->d_RY};
    memset(S->h_loc + ni * rec, 0, sizeof(double) * rec * ((size_t)S->nrec - ni));
    for (int q = 0; q < 4; q++)
        TRY(spk_memcpy_2d(S->h_loc + q * TS, sizeof(double) * rec, src[q], sizeof(double) * TS, sizeof(double) * TS,
                          ni, S->c->stream));
    return spk_stream_sync(S->c->stream);
}

/* rank 0: the global records -> the global reduced plan's blocks */
static int unpack_blocks(shard_t *S)
{
    const size_t TS = (size_t)S->KB * S->KB, ng = (size_t)S->p - 1, rec = 4 * TS;
    spk_plan *G = S->Pg;
    void *dst[4] = {G->d_RP, G->d_RX, G->d_RQ, G->d_RY};
    for (int q = 0; q < 4; q++)
        TRY(spk_memcpy_2d(dst[q], sizeof(double) * TS, S->h_glob + q * TS, sizeof(double) * rec, sizeof(double) * TS,
                          ng, S->c->stream));
    return spk_stream_sync(S->c->stream);
}

/* reduced right-hand side / solution, device layout [column][interface][2 KB]
 * (bottom tip of the left partition, then top tip of the right one) <-> records
 * [interface]{b: [column][KB], t: [column][KB]} */
static void red_to_records(const double *dev, int nif, int KB, int nr, double *recs)
{
    const size_t NR = (size_t)nif * 2 * KB, rec = (size_t)2 * KB * nr;
    for (int j = 0; j < nif; j++)
        for (int hh = 0; hh < nr; hh++) {
            const double *s = dev + (size_t)hh * NR + (size_t)j * 2 * KB;
            memcpy(recs + (size_t)j * rec + (size_t)hh * KB, s, sizeof(double) * KB);
            memcpy(recs + (size_t)j * rec + (size_t)(nr + hh) * KB, s + KB, sizeof(double) * KB);
        }
}
static void records_to_red(const double *recs, int nif, int KB, int nr, double *dev)
{
    const size_t NR = (size_t)nif * 2 * KB, rec = (size_t)2 * KB * nr;
    for (int j = 0; j < nif; j++)
        for (int hh = 0; hh < nr; hh++) {
            double *d = dev + (size_t)hh * NR + (size_t)j * 2 * KB;
            memcpy(d, recs + (size_t)j * rec + (size_t)hh * KB, sizeof(double) * KB);
            memcpy(d + KB, recs + (size_t)j * rec + (size_t)(nr + hh) * KB, sizeof(double) * KB);
        }
}

/* one SPIKE application over all ranks: x (+)= A^{-1} rhs */
static int shard_apply(shard_t *S, const double *d_rhs, int accumulate, int red_refine, int *peer)
{
    const spike_comm_t *cm = S->cm;
    const int KB = S->KB, nr = S->nrhs, nl = S->nloc_if, rec = 2 * KB * nr;
    void *st = S->c->stream;
    int rc = spk_apply(S->P, d_rhs, nr, st);
    const size_t NRl = (size_t)nl * 2 * KB;
    if (rc == SPK_OK) rc = spk_memcpy_d2h(S->h_dev, S->P->d_g, sizeof(double) * NRl * nr, st);
    if (rc == SPK_OK) rc = spk_stream_sync(st);
    rc = agree(S, rc, peer);
    if (rc != SPK_OK) return rc;
    memset(S->h_loc, 0, sizeof(double) * (size_t)rec * S->nrec);
    red_to_records(S->h_dev, nl, KB, nr, S->h_loc);
    const size_t slot = sizeof(double) * (size_t)rec * S->nrec;
    if (cm->gather(cm->user, S->h_loc, slot, S->h_all) != 0) return SPK_ECUDA;
    rc = SPK_OK;
    if (cm->rank == 0) {
        spk_plan *G = S->Pg;
        const int ng = S->p - 1;
        spike_shard_assemble(S->p, cm->size, KB * nr, KB * nr, S->h_all, S->h_glob);
        records_to_red(S->h_glob, ng, KB, nr, S->h_dev);
        rc = spk_memcpy_h2d(G->d_g, S->h_dev, sizeof(double) * (size_t)ng * 2 * KB * nr, st);
        if (rc == SPK_OK) rc = spk_reduced_solve(G, nr, red_refine, st);
        if (rc == SPK_OK) rc = spk_memcpy_d2h(S->h_dev, G->d_u, sizeof(double) * (size_t)ng * 2 * KB * nr, st);
        if (rc == SPK_OK) rc = spk_stream_sync(st);
        if (rc == SPK_OK) {
            red_to_records(S->h_dev, ng, KB, nr, S->h_glob);
            spike_shard_split(S->p, cm->size, KB * nr, KB * nr, S->h_glob, S->h_all);
        }
    }
    rc = agree(S, rc, peer);
    if (rc != SPK_OK) return rc;
    if (cm->scatter(cm->user, S->h_all, slot, S->h_loc) != 0) return SPK_ECUDA;
    records_to_red(S->h_loc, nl, KB, nr, S->h_dev);
    rc = spk_memcpy_h2d(S->P->d_u, S->h_dev, sizeof(double) * NRl * nr, st);
    if (rc == SPK_OK) rc = spk_retrieve(S->P, S->d_x, nr, accumulate, st);
    if (rc == SPK_OK) rc = spk_stream_sync(st);
    return agree(S, rc, peer);
}

/* KB rows of x with each neighbour into the halo rows (and b's halo rows set
 * to the same values, so the halo rows' residual is zero) */
static int shard_halo(shard_t *S, int *peer)
{
    const spike_comm_t *cm = S->cm;
    const int KB = S->KB, h = S->h, m = S->rows, nl = S->n_loc, nr = S->nrhs;
    const size_t blk = (size_t)KB * nr;
    double *to_lo = S->h_halo, *to_hi = to_lo + blk, *from_lo = to_hi + blk, *from_hi = from_lo + blk;
    void *st = S->c->stream;
    int rc = SPK_OK;
    for (int k = 0; k < nr && rc == SPK_OK; k++) {
        rc = spk_memcpy_d2h(to_lo + (size_t)k * KB, S->d_x + (size_t)k * nl + h, sizeof(double) * KB, st);
        if (rc == SPK_OK)
            rc = spk_memcpy_d2h(to_hi + (size_t)k * KB, S->d_x + (size_t)k * nl + h + m - KB, sizeof(double) * KB, st);
    }
    if (rc == SPK_OK) rc = spk_stream_sync(st);
    rc = agree(S, rc, peer);
    if (rc != SPK_OK) return rc;
    memset(from_lo, 0, sizeof(double) * 2 * blk);
    if (cm->exchange(cm->user, to_lo, to_hi, from_lo, from_hi, sizeof(double) * blk) != 0) return SPK_ECUDA;
    for (int k = 0; k < nr && rc == SPK_OK; k++) {
        double *xl = S->d_x + (size_t)k * nl, *bl = S->d_b + (size_t)k * nl;
        if (cm->rank > 0) {
            rc = spk_memcpy_h2d(xl + h - KB, from_lo + (size_t)k * KB, sizeof(double) * KB, st);
            if (rc == SPK_OK) rc = spk_memcpy_h2d(bl + h - KB, from_lo + (size_t)k * KB, sizeof(double) * KB, st);
        }
        if (rc == SPK_OK && cm->rank < cm->size - 1) {
            rc = spk_memcpy_h2d(xl + h + m, from_hi + (size_t)k * KB, sizeof(double) * KB, st);
            if (rc == SPK_OK) rc = spk_memcpy_h2d(bl + h + m, from_hi + (size_t)k * KB, sizeof(double) * KB, st);
        }
    }
    if (rc == SPK_OK) rc = spk_stream_sync(st);
    return agree(S, rc, peer);
}

static Error_t shard_fail(int rc, int peer, const char *name)
{
    if (peer) return spk_fail(SPIKE_ERR_CUDA, "%s: another rank failed (error code %d there)", name, rc);
    if (rc == SPK_ECONV) return spk_fail(SPIKE_ERR_CONVERGENCE, "%s: refinement stopped above the tolerance", name);
    return spk_fail_code(rc, name);
}

Error_t spike_shard_dsolve(spike_context_t ctx, const spike_comm_t *cm, integer_t n, integer_t p, integer_t nrhs,
                           integer_t rows, integer_t nnz, const integer_t *colind, const integer_t *rowptr,
                           const double *aij, double *x, const double *b)
{
    const char *name = "spike_shard_dsolve";
    if (!cm || !cm->gather || !cm->scatter || !cm->allreduce_sum || !cm->exchange || cm->size < 1 || cm->rank < 0 ||
        cm->rank >= cm->size)
        return spk_fail(SPIKE_ERR_ARGUMENT, "%s: incomplete communicator", name);
    if (nrhs < 1 || nrhs > RHS_CHUNK) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: nrhs must be in [1, %d]", name, RHS_CHUNK);
    if (p < 2 || cm->size > p) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: need p >= 2 and at most p ranks", name);
    int part0, part1, row0, row1;
    if (spike_shard_range(n, p, cm->size, cm->rank, &part0, &part1, &row0, &row1) != SPIKE_SUCCESS) return SPIKE_ERROR;
    int rc = SPK_OK, peer = 0;
    if (rows != row1 - row0 || nnz < 0 || !colind || !rowptr || !aij || !x || !b || rowptr[0] != 0 ||
        rowptr[rows] != nnz)
        rc = SPK_EARG;
    spike_context_t c = rc == SPK_OK ? spk_get_ctx(ctx) : NULL;
    if (rc == SPK_OK && !c) rc = SPK_ENODEV;
    shard_t *S = NULL;
    if (rc == SPK_OK) rc = shard_buffers(c, cm, n, p, nrhs, rows, nnz, part0, part1, row0, &S);
    if (S) {
        S->cm = cm;
        S->c = c;
    }
    /* bandwidth of this rank's rows (global numbering), then of all ranks'
     * (each writes its own pair of slots of a vector summed over the ranks),
     * and ||b||^2 per column summed the same way */
    const int size = cm->size;
    const int nv = 2 * size + nrhs + 1;
    double *v = (double *)calloc((size_t)nv, sizeof(double));
    if (!v) rc = SPK_EMEM;
    int copying = 0;
    if (rc == SPK_OK) {
        /* the rank's rows to the device: row pointers and columns first (the
         * band scan reads them), the values behind them on the copy stream,
         * where they overlap the scan and the agreement on the block size */
        const size_t H = SHARD_HALO_MAX;
        int *rp_raw = S->d_rp_buf + H, *ci_raw = S->d_ci_buf + H;
        rc = spk_memcpy_h2d(rp_raw, rowptr, sizeof(int) * ((size_t)rows + 1), c->stream);
        if (rc == SPK_OK && nnz > 0) rc = spk_memcpy_h2d(ci_raw, colind, sizeof(int) * (size_t)nnz, c->stream);
        if (rc == SPK_OK && !c->copy_stream) rc = spk_stream_create(&c->copy_stream);
        if (rc == SPK_OK) rc = spk_stream_fork(c->stream, c->copy_stream);
        if (rc == SPK_OK && nnz > 0) {
            copying = 1;
            rc = spk_memcpy_h2d(S->d_a_buf + H, aij, sizeof(double) * (size_t)nnz, c->copy_stream);
        }
        if (rc == SPK_OK) rc = spk_rows_band(rows, nnz, row0, n, rp_raw, ci_raw, c->d_scratch, c->stream);
        for (int k = 0; k < nrhs; k++)
            for (int r = 0; r < rows; r++) v[2 * size + k] += b[(size_t)k * rows + r] * b[(size_t)k * rows + r];
        int band[3] = {0, 0, 0};
        if (rc == SPK_OK) rc = spk_memcpy_d2h(band, c->d_scratch, sizeof band, c->stream);
        if (rc == SPK_OK) rc = spk_stream_sync(c->stream);
        if (rc == SPK_OK && band[2]) rc = SPK_ECSR;
        v[2 * cm->rank] = band[0];
        v[2 * cm->rank + 1] = band[1];
    }
    if (copying) { /* everything after this on the context's stream sees the values */
        const int jrc = spk_stream_fork(c->copy_stream, c->stream);
        if (rc == SPK_OK) rc = jrc;
    }
    if (v) {
        v[nv - 1] = rc != SPK_OK;
        if (cm->allreduce_sum(cm->user, v, nv) != 0) rc = SPK_ECUDA;
        else if (v[nv - 1] != 0 && rc == SPK_OK) {
            rc = SPK_EARG;
            peer = 1;
        }
    }
    double bnorm[RHS_CHUNK];
    int KB = 0;
    if (rc == SPK_OK) {
        int k = 0;
        for (int r = 0; r < size; r++) {
            if (v[2 * r] > k) k = (int)v[2 * r];
            if (v[2 * r + 1] > k) k = (int)v[2 * r + 1];
        }
        for (int j = 0; j < nrhs; j++) bnorm[j] = sqrt(v[2 * size + j]);
        KB = spk_choose_block(k < 1 ? 1 : k);
        if (!KB || spk_factor_smem(KB, 0, c->mode) == 0) rc = SPK_EBAND;
        /* every partition must hold two tiles (all ranks decide alike) */
        else if (n / p < 2 * KB)
            rc = SPK_EARG;
    }
    free(v);
    if (rc != SPK_OK) {
        spk_shard_release(c);
        if (rc == SPK_EARG && !peer)
            return spk_fail(SPIKE_ERR_ARGUMENT, "%s: bad arguments (rows must be this rank's range, rowptr from 0 to "
                            "nnz, partitions at least two tiles long)", name);
        return shard_fail(rc, peer, name);
    }
    const size_t TS = (size_t)KB * KB, rec_blk = 4 * TS;

    /* local system, factorization, interface blocks */
    rc = shard_plans(S, KB);
    if (rc == SPK_OK) rc = shard_local(S, b);
    if (rc == SPK_OK) {
        int info[3];
        long long l0 = 0;
        rc = spk_analyze(S->n_loc, S->nnz_loc, S->d_rp, S->d_ci, c->d_scratch, info, c->stream, &l0);
        if (rc == SPK_OK && info[2]) rc = SPK_ECSR;
    }
    if (rc == SPK_OK) {
        S->P->twist = S->P->twist_cap && c->twist;
        S->P->red_fp64 = c->red_fp64 && KB <= 64;
        rc = spk_memset(S->P->d_err, 0, sizeof(unsigned) * 4, c->stream);
        if (rc == SPK_OK) rc = spk_factor(S->P, S->d_rp, S->d_ci, S->d_a, c->stream);
        if (rc == SPK_OK) rc = device_error(S->P, c->stream);
    }
    if (rc == SPK_OK) rc = pack_blocks(S);
    rc = agree(S, rc, &peer);
    if (rc == SPK_OK && cm->gather(cm->user, S->h_loc, sizeof(double) * rec_blk * S->nrec, S->h_all) != 0)
        rc = SPK_ECUDA;
    if (rc == SPK_OK) {
        int rc0 = SPK_OK;
        if (cm->rank == 0) {
            spk_plan *G = S->Pg;
            G->red_fp64 = c->red_fp64 && KB <= 64;
            rc0 = spike_shard_assemble(p, size, 2 * TS, 2 * TS, S->h_all, S->h_glob) == SPIKE_SUCCESS ? SPK_OK : SPK_EARG;
            if (rc0 == SPK_OK) rc0 = unpack_blocks(S);
            if (rc0 == SPK_OK) rc0 = spk_memset(G->d_err, 0, sizeof(unsigned) * 4, c->stream);
            if (rc0 == SPK_OK) rc0 = spk_reduced_factor(G, c->stream);
            if (rc0 == SPK_OK) rc0 = device_error(G, c->stream);
        }
        rc = agree(S, rc0, &peer);
    }

    /* solve and FP64 refinement */
    const int red = c->red_refine > 0 ? c->red_refine : (c->mode == SPK_MIXED && !(c->red_fp64 && KB <= 64) ? 2 : 1);
    double relres = 0.0;
    int sweeps = 0;
    if (rc == SPK_OK) rc = shard_apply(S, S->d_b, 0, red, &peer);
    for (int sweep = 0; rc == SPK_OK; sweep++) {
        rc = shard_halo(S, &peer);
        if (rc != SPK_OK) break;
        double nrm[RHS_CHUNK + 1];
        int lrc = spk_residual(S->P, S->d_rp, S->d_ci, S->d_a, S->d_x, S->d_b, S->d_r, nrhs, 0, S->P->d_norms,
                               c->stream);
        if (lrc == SPK_OK) lrc = spk_memcpy_d2h(nrm, S->P->d_norms, sizeof(double) * nrhs, c->stream);
        if (lrc == SPK_OK) lrc = spk_stream_sync(c->stream);
        rc = agree(S, lrc, &peer);
        if (rc != SPK_OK) break;
        if (cm->allreduce_sum(cm->user, nrm, nrhs) != 0) {
            rc = SPK_ECUDA;
            break;
        }
        double worst = 0.0;
        for (int j = 0; j < nrhs; j++) {
            const double rel = sqrt(nrm[j]) / (bnorm[j] > 0 ? bnorm[j] : 1.0);
            if (!(rel <= worst)) worst = rel;
        }
        relres = worst;
        sweeps = sweep;
        if (worst <= c->tol) break;
        if (sweep >= c->max_refine) {
            rc = SPK_ECONV;
            break;
        }
        rc = shard_apply(S, S->d_r, 1, red, &peer);
    }
    if (rc == SPK_OK || rc == SPK_ECONV) {
        int lrc = SPK_OK;
        for (int k = 0; k < nrhs && lrc == SPK_OK; k++)
            lrc = spk_memcpy_d2h(x + (size_t)k * rows, S->d_x + (size_t)k * S->n_loc + S->h, sizeof(double) * rows,
                                 c->stream);
        if (lrc == SPK_OK) lrc = spk_stream_sync(c->stream);
        if (lrc != SPK_OK) rc = lrc;
        c->info.relres_max = relres;
        c->info.refine_sweeps = sweeps;
        c->info.partitions = p;
        c->info.block = KB;
        c->info.twisted = S->P->twist;
        c->info.columns_implied = 0;
        c->info.reduced_fp64 = (c->red_fp64 && KB <= 64) || c->mode == SPK_PLAIN;
    }
    /* a failed call leaves nothing behind for the next one */
    if (rc != SPK_OK && rc != SPK_ECONV) spk_shard_release(c);
    if (rc == SPK_OK) return spk_succeed();
    return shard_fail(rc, peer, name);
}
