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
typedef struct {
    const spike_comm_t *cm;
    spike_context_t c;
    int n, p, nrhs, rows, part0, part1, row0, KB, h, nloc_if, nrec;
    long long nnz;
    /* local system */
    int n_loc;
    long long nnz_loc;
    spk_plan *P;  /* the local system's plan */
    spk_plan *Pg; /* rank 0: the global reduced system */
    int *d_rp, *d_ci;
    double *d_a, *d_b, *d_x, *d_r;
    /* host staging */
    double *h_loc;   /* this rank's slot */
    double *h_all;   /* rank 0: every rank's slot */
    double *h_glob;  /* rank 0: the global records */
    double *h_dev;   /* device-layout staging (interface blocks or reduced right-hand side) */
    double *h_halo;  /* 4 KB x nrhs: to lo, to hi, from lo, from hi */
} shard_t;

static void shard_free(shard_t *S)
{
    spk_plan_destroy(S->P);
    spk_plan_destroy(S->Pg);
    spk_free(S->d_rp);
    spk_free(S->d_ci);
    spk_free(S->d_a);
    spk_free(S->d_b);
    spk_free(S->d_x);
    spk_free(S->d_r);
    free(S->h_loc);
    free(S->h_all);
    free(S->h_glob);
    free(S->h_dev);
    free(S->h_halo);
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

/* This rank's rows renumbered with h identity rows on either side, on the
 * device, with the local schedule: halo partition, the rank's partitions,
 * halo partition. */
static int shard_local(shard_t *S, const int *colind, const int *rowptr, const double *aij, const double *b)
{
    const int h = S->h, m = S->rows, nl = m + 2 * h;
    S->n_loc = nl;
    S->nnz_loc = S->nnz + 2LL * h;
    int *rp = (int *)malloc(sizeof(int) * ((size_t)nl + 1));
    int *ci = (int *)malloc(sizeof(int) * (size_t)S->nnz_loc);
    double *a = (double *)malloc(sizeof(double) * (size_t)S->nnz_loc);
    double *bl = (double *)calloc((size_t)nl * S->nrhs, sizeof(double));
    const int np = S->part1 - S->part0, pl = np + 2;
    int *ps = (int *)malloc(sizeof(int) * ((size_t)pl + 1));
    int rc = (rp && ci && a && bl && ps) ? SPK_OK : SPK_EMEM;
    if (rc == SPK_OK) {
        long long t = 0;
        for (int i = 0; i < h; i++, t++) {
            rp[i] = (int)t;
            ci[t] = i;
            a[t] = 1.0;
        }
        for (int r = 0; r < m && rc == SPK_OK; r++) {
            rp[h + r] = (int)t;
            for (long long q = rowptr[r]; q < rowptr[r + 1]; q++, t++) {
                const long long cl = (long long)colind[q] - S->row0 + h;
                if (cl < 0 || cl >= nl) { /* farther than the halo reaches: not a band of <= KB */
                    rc = SPK_ECSR;
                    break;
                }
                ci[t] = (int)cl;
                a[t] = aij[q];
            }
        }
        for (int i = 0; rc == SPK_OK && i < h; i++, t++) {
            rp[h + m + i] = (int)t;
            ci[t] = h + m + i;
            a[t] = 1.0;
        }
        rp[nl] = (int)t;
        for (int k = 0; k < S->nrhs; k++) memcpy(bl + (size_t)k * nl + h, b + (size_t)k * m, sizeof(double) * m);
        ps[0] = 0;
        for (int j = 0; j <= np; j++) ps[1 + j] = h + (int)(part_row(S->n, S->p, S->part0 + j) - S->row0);
        ps[pl] = nl;
    }
    if (rc == SPK_OK)
        rc = spk_plan_build(nl, S->nnz_loc, S->KB, S->KB, S->KB, 0, S->c->mode, pl, ps, S->nrhs, S->c->stream, 0, &S->P);
    const size_t vb = sizeof(double) * (size_t)nl * S->nrhs;
    if (rc == SPK_OK) rc = spk_malloc((void **)&S->d_rp, sizeof(int) * ((size_t)nl + 1));
    if (rc == SPK_OK) rc = spk_malloc((void **)&S->d_ci, sizeof(int) * (size_t)S->nnz_loc);
    if (rc == SPK_OK) rc = spk_malloc((void **)&S->d_a, sizeof(double) * (size_t)S->nnz_loc);
    if (rc == SPK_OK) rc = spk_malloc((void **)&S->d_b, vb);
    if (rc == SPK_OK) rc = spk_malloc((void **)&S->d_x, vb);
    if (rc == SPK_OK) rc = spk_malloc((void **)&S->d_r, vb);
    void *st = S->c->stream;
    if (rc == SPK_OK) rc = spk_memcpy_h2d(S->d_rp, rp, sizeof(int) * ((size_t)nl + 1), st);
    if (rc == SPK_OK) rc = spk_memcpy_h2d(S->d_ci, ci, sizeof(int) * (size_t)S->nnz_loc, st);
    if (rc == SPK_OK) rc = spk_memcpy_h2d(S->d_a, a, sizeof(double) * (size_t)S->nnz_loc, st);
    if (rc == SPK_OK) rc = spk_memcpy_h2d(S->d_b, bl, vb, st);
    if (rc == SPK_OK) rc = spk_memset(S->d_x, 0, vb, st);
    if (rc == SPK_OK) rc = spk_stream_sync(st);
    free(rp);
    free(ci);
    free(a);
    free(bl);
    free(ps);
    return rc;
}

/* Local interface j's record of the interface blocks: P X (bottom tips of its
 * left partition) | Q Y (top tips of its right partition), KB x KB each. */
static int pack_blocks(shard_t *S)
{
    const size_t TS = (size_t)S->KB * S->KB, ni = (size_t)S->nloc_if, rec = 4 * TS;
    spk_plan *P = S->P;
    double *blk[4] = {S->h_dev, S->h_dev + ni * TS, S->h_dev + 2 * ni * TS, S->h_dev + 3 * ni * TS};
    void *src[4] = {P->d_RP, P->d_RX, P->d_RQ, P->d_RY};
    for (int q = 0; q < 4; q++) TRY(spk_memcpy_d2h(blk[q], src[q], sizeof(double) * ni * TS, S->c->stream));
    TRY(spk_stream_sync(S->c->stream));
    memset(S->h_loc, 0, sizeof(double) * rec * S->nrec);
    for (size_t j = 0; j < ni; j++)
        for (int q = 0; q < 4; q++) memcpy(S->h_loc + j * rec + q * TS, blk[q] + j * TS, sizeof(double) * TS);
    return SPK_OK;
}

/* rank 0: the global records -> the global reduced plan's blocks */
static int unpack_blocks(shard_t *S)
{
    const size_t TS = (size_t)S->KB * S->KB, ng = (size_t)S->p - 1, rec = 4 * TS;
    spk_plan *G = S->Pg;
    void *dst[4] = {G->d_RP, G->d_RX, G->d_RQ, G->d_RY};
    for (int q = 0; q < 4; q++) {
        for (size_t g = 0; g < ng; g++) memcpy(S->h_dev + g * TS, S->h_glob + g * rec + q * TS, sizeof(double) * TS);
        TRY(spk_memcpy_h2d(dst[q], S->h_dev, sizeof(double) * ng * TS, S->c->stream));
        TRY(spk_stream_sync(S->c->stream));
    }
    return SPK_OK;
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
    shard_t S;
    memset(&S, 0, sizeof S);
    S.cm = cm;
    S.n = n;
    S.p = p;
    S.nrhs = nrhs;
    S.rows = rows;
    S.nnz = nnz;
    int part0, part1, row0, row1;
    if (spike_shard_range(n, p, cm->size, cm->rank, &part0, &part1, &row0, &row1) != SPIKE_SUCCESS) return SPIKE_ERROR;
    S.part0 = part0;
    S.part1 = part1;
    S.row0 = row0;
    int rc = SPK_OK, peer = 0;
    if (rows != row1 - row0 || nnz < 0 || !colind || !rowptr || !aij || !x || !b || rowptr[0] != 0 ||
        rowptr[rows] != nnz)
        rc = SPK_EARG;
    spike_context_t c = rc == SPK_OK ? spk_get_ctx(ctx) : NULL;
    if (rc == SPK_OK && !c) rc = SPK_ENODEV;
    S.c = c;
    /* bandwidth of this rank's rows (global numbering), then of all ranks'
     * (each writes its own pair of slots of a vector summed over the ranks),
     * and ||b||^2 per column summed the same way */
    const int size = cm->size;
    const int nv = 2 * size + nrhs + 1;
    double *v = (double *)calloc((size_t)nv, sizeof(double));
    if (!v) rc = SPK_EMEM;
    if (rc == SPK_OK) {
        int ku = 0, kl = 0;
        for (int r = 0; r < rows && rc == SPK_OK; r++)
            for (long long q = rowptr[r]; q < rowptr[r + 1]; q++) {
                const long long col = colind[q], d = col - (row0 + r);
                if (col < 0 || col >= n || q < 0 || q >= nnz) {
                    rc = SPK_ECSR;
                    break;
                }
                if (d > ku) ku = (int)d;
                if (-d > kl) kl = (int)-d;
            }
        v[2 * cm->rank] = ku;
        v[2 * cm->rank + 1] = kl;
        for (int k = 0; k < nrhs; k++)
            for (int r = 0; r < rows; r++) v[2 * size + k] += b[(size_t)k * rows + r] * b[(size_t)k * rows + r];
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
    if (rc == SPK_OK) {
        int k = 0;
        for (int r = 0; r < size; r++) {
            if (v[2 * r] > k) k = (int)v[2 * r];
            if (v[2 * r + 1] > k) k = (int)v[2 * r + 1];
        }
        for (int j = 0; j < nrhs; j++) bnorm[j] = sqrt(v[2 * size + j]);
        S.KB = spk_choose_block(k < 1 ? 1 : k);
        if (!S.KB || spk_factor_smem(S.KB, 0, c->mode) == 0) rc = SPK_EBAND;
        /* every partition must hold two tiles (all ranks decide alike) */
        else if (n / p < 2 * S.KB)
            rc = SPK_EARG;
    }
    free(v);
    if (rc != SPK_OK) {
        if (rc == SPK_EARG && !peer)
            return spk_fail(SPIKE_ERR_ARGUMENT, "%s: bad arguments (rows must be this rank's range, rowptr from 0 to "
                            "nnz, partitions at least two tiles long)", name);
        return shard_fail(rc, peer, name);
    }
    S.h = 8 * S.KB;
    S.nloc_if = (part1 - part0) + 1;
    S.nrec = slot_records(p, size);
    const int KB = S.KB;
    const size_t TS = (size_t)KB * KB;
    const size_t rec_blk = 4 * TS, rec_red = (size_t)2 * KB * nrhs;
    const size_t rec_max = rec_blk > rec_red ? rec_blk : rec_red;
    S.h_loc = (double *)malloc(sizeof(double) * rec_max * S.nrec);
    S.h_dev = (double *)malloc(sizeof(double) * rec_max * (size_t)(p > S.nrec ? p : S.nrec));
    S.h_halo = (double *)malloc(sizeof(double) * 4 * (size_t)KB * nrhs);
    if (cm->rank == 0) {
        S.h_all = (double *)malloc(sizeof(double) * rec_max * S.nrec * (size_t)size);
        S.h_glob = (double *)malloc(sizeof(double) * rec_max * (size_t)p);
    }
    if (!S.h_loc || !S.h_dev || !S.h_halo || (cm->rank == 0 && (!S.h_all || !S.h_glob))) rc = SPK_EMEM;

    /* local system, factorization, interface blocks */
    if (rc == SPK_OK) rc = shard_local(&S, colind, rowptr, aij, b);
    if (rc == SPK_OK) {
        int info[3];
        long long l0 = 0;
        rc = spk_analyze(S.n_loc, S.nnz_loc, S.d_rp, S.d_ci, c->d_scratch, info, c->stream, &l0);
        if (rc == SPK_OK && info[2]) rc = SPK_ECSR;
    }
    if (rc == SPK_OK) {
        S.P->twist = S.P->twist_cap && c->twist;
        S.P->red_fp64 = c->red_fp64 && KB <= 64;
        rc = spk_memset(S.P->d_err, 0, sizeof(unsigned) * 4, c->stream);
        if (rc == SPK_OK) rc = spk_factor(S.P, S.d_rp, S.d_ci, S.d_a, c->stream);
        if (rc == SPK_OK) rc = device_error(S.P, c->stream);
    }
    if (rc == SPK_OK) rc = pack_blocks(&S);
    rc = agree(&S, rc, &peer);
    if (rc == SPK_OK && cm->gather(cm->user, S.h_loc, sizeof(double) * rec_blk * S.nrec, S.h_all) != 0) rc = SPK_ECUDA;
    if (rc == SPK_OK) {
        int rc0 = SPK_OK;
        if (cm->rank == 0) {
            rc0 = spk_plan_reduced_build(p, KB, 0, c->mode, nrhs, &S.Pg);
            if (rc0 == SPK_OK) S.Pg->red_fp64 = c->red_fp64 && KB <= 64;
            if (rc0 == SPK_OK) rc0 = spike_shard_assemble(p, size, 2 * TS, 2 * TS, S.h_all, S.h_glob) == SPIKE_SUCCESS
                                         ? SPK_OK : SPK_EARG;
            if (rc0 == SPK_OK) rc0 = unpack_blocks(&S);
            if (rc0 == SPK_OK) rc0 = spk_memset(S.Pg->d_err, 0, sizeof(unsigned) * 4, c->stream);
            if (rc0 == SPK_OK) rc0 = spk_reduced_factor(S.Pg, c->stream);
            if (rc0 == SPK_OK) rc0 = device_error(S.Pg, c->stream);
        }
        rc = agree(&S, rc0, &peer);
    }

    /* solve and FP64 refinement */
    const int red = c && c->red_refine > 0 ? c->red_refine : (c && c->mode == SPK_MIXED && !(c->red_fp64 && KB <= 64) ? 2 : 1);
    double relres = 0.0;
    int sweeps = 0;
    if (rc == SPK_OK) rc = shard_apply(&S, S.d_b, 0, red, &peer);
    for (int sweep = 0; rc == SPK_OK; sweep++) {
        rc = shard_halo(&S, &peer);
        if (rc != SPK_OK) break;
        double nrm[RHS_CHUNK + 1];
        int lrc = spk_residual(S.P, S.d_rp, S.d_ci, S.d_a, S.d_x, S.d_b, S.d_r, nrhs, 0, S.P->d_norms, c->stream);
        if (lrc == SPK_OK) lrc = spk_memcpy_d2h(nrm, S.P->d_norms, sizeof(double) * nrhs, c->stream);
        if (lrc == SPK_OK) lrc = spk_stream_sync(c->stream);
        rc = agree(&S, lrc, &peer);
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
        rc = shard_apply(&S, S.d_r, 1, red, &peer);
    }
    if (rc == SPK_OK || rc == SPK_ECONV) {
        int lrc = SPK_OK;
        for (int k = 0; k < nrhs && lrc == SPK_OK; k++)
            lrc = spk_memcpy_d2h(x + (size_t)k * rows, S.d_x + (size_t)k * S.n_loc + S.h, sizeof(double) * rows,
                                 c->stream);
        if (lrc == SPK_OK) lrc = spk_stream_sync(c->stream);
        if (lrc != SPK_OK) rc = lrc;
        c->info.relres_max = relres;
        c->info.refine_sweeps = sweeps;
        c->info.partitions = p;
        c->info.block = KB;
        c->info.twisted = S.P ? S.P->twist : 0;
        c->info.columns_implied = 0;
        c->info.reduced_fp64 = (c->red_fp64 && KB <= 64) || c->mode == SPK_PLAIN;
    }
    shard_free(&S);
    if (rc == SPK_OK) return spk_succeed();
    return shard_fail(rc, peer, name);
}
