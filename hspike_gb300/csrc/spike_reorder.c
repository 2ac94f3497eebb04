/*
 * spike_reorder.c -- bandwidth-reducing reordering for general sparse inputs.
 *
 * The reference reorders with cuSolverSp's host RCM and permutes the CSR with
 * csrperm (cuda_standalone_symrcm, OpenMP/spike_cuda.c:898-971), and permutes
 * vectors Matlab-style (permute_vector, OpenMP/spike_algebra.c:34-53; its
 * reorder_rcm at :23-30 is a stub).  Here, in plain C on the host:
 *
 *   spike_rcm_permutation  reverse Cuthill-McKee on the pattern of A + A^T:
 *                          each connected component starts from a
 *                          pseudo-peripheral node (George & Liu's iteration:
 *                          BFS from a minimum-degree node, restart from the
 *                          minimum-degree node of the last level while the
 *                          eccentricity grows), visits neighbours in
 *                          increasing degree, and the order is reversed;
 *   spike_permute_csr      B = A(p, p), rows sorted by column;
 *   spike_permute_vector   v = v(p) (flag > 0) or v(p) = v (flag <= 0), for
 *                          nrhs columns of length n;
 *   spike_dsolve_reordered permute, solve on the device, permute back.
 */
#include <stdlib.h>
#include <string.h>

#include "spike_host_internal.h"

/* symmetric adjacency of the pattern, diagonal dropped, duplicates merged */
static int sym_graph(int n, const int *rp, const int *ci, int **xadj_out, int **adj_out)
{
    int *deg = (int *)calloc((size_t)n + 1, sizeof(int));
    if (!deg) return SPK_EMEM;
    for (int r = 0; r < n; r++)
        for (int t = rp[r]; t < rp[r + 1]; t++) {
            const int c = ci[t];
            if (c == r) continue;
            deg[r]++;
            deg[c]++;
        }
    int *xadj = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    long long tot = 0;
    for (int r = 0; r < n; r++) tot += deg[r];
    int *adj = (int *)malloc(sizeof(int) * (size_t)(tot > 0 ? tot : 1));
    if (!xadj || !adj) {
        free(deg);
        free(xadj);
        free(adj);
        return SPK_EMEM;
    }
    xadj[0] = 0;
    for (int r = 0; r < n; r++) xadj[r + 1] = xadj[r] + deg[r];
    memset(deg, 0, sizeof(int) * (size_t)n);
    for (int r = 0; r < n; r++)
        for (int t = rp[r]; t < rp[r + 1]; t++) {
            const int c = ci[t];
            if (c == r) continue;
            adj[xadj[r] + deg[r]++] = c;
            adj[xadj[c] + deg[c]++] = r;
        }
    /* sort and merge each list (insertion sort: lists are short for banded
     * inputs; a mark array merges duplicates) */
    int *mark = (int *)malloc(sizeof(int) * (size_t)n);
    if (!mark) {
        free(deg);
        free(xadj);
        free(adj);
        return SPK_EMEM;
    }
    for (int i = 0; i < n; i++) mark[i] = -1;
    int w = 0;
    for (int r = 0; r < n; r++) {
        const int b = xadj[r], e = xadj[r] + deg[r];
        const int start = w;
        for (int t = b; t < e; t++) {
            const int c = adj[t];
            if (mark[c] == r) continue;
            mark[c] = r;
            int k = w++;
            while (k > start && adj[k - 1] > c) {
                adj[k] = adj[k - 1];
                k--;
            }
            adj[k] = c;
        }
        xadj[r] = start;
    }
    xadj[n] = w;
    free(mark);
    free(deg);
    *xadj_out = xadj;
    *adj_out = adj;
    return SPK_OK;
}

/* BFS from `root`: returns the number of levels; queue[0..*qlen) holds the
 * visit order (level by level) and the last level starts at *last_begin */
static int bfs_levels(int root, const int *xadj, const int *adj, int *level, int *queue, int stamp, int *seen,
                      int *last_begin, int *qlen)
{
    int head = 0, tail = 0, nl = 0;
    queue[tail++] = root;
    seen[root] = stamp;
    level[root] = 0;
    *last_begin = 0;
    while (head < tail) {
        const int v = queue[head++];
        if (level[v] + 1 > nl) {
            nl = level[v] + 1;
            *last_begin = head - 1;
        }
        for (int t = xadj[v]; t < xadj[v + 1]; t++) {
            const int u = adj[t];
            if (seen[u] == stamp) continue;
            seen[u] = stamp;
            level[u] = level[v] + 1;
            queue[tail++] = u;
        }
    }
    *qlen = tail;
    return nl;
}

Error_t spike_rcm_permutation(integer_t n, integer_t nnz, const integer_t *colind, const integer_t *rowptr,
                              integer_t *perm)
{
    if (n < 0 || nnz < 0 || !perm || (n > 0 && (!colind || !rowptr)))
        return spk_fail(SPIKE_ERR_ARGUMENT, "spike_rcm_permutation: bad argument");
    if (n == 0) return spk_succeed();
    for (int r = 0; r < n; r++)
        if (rowptr[r] < 0 || rowptr[r + 1] < rowptr[r] || rowptr[r + 1] > nnz)
            return spk_fail(SPIKE_ERR_CSR, "spike_rcm_permutation: invalid row pointers");
    for (int t = 0; t < nnz; t++)
        if (colind[t] < 0 || colind[t] >= n) return spk_fail(SPIKE_ERR_CSR, "spike_rcm_permutation: column out of range");
    int *xadj = NULL, *adj = NULL;
    if (sym_graph(n, rowptr, colind, &xadj, &adj) != SPK_OK)
        return spk_fail(SPIKE_ERR_MEMORY, "spike_rcm_permutation: host allocation failed");
    int *level = (int *)malloc(sizeof(int) * (size_t)n);
    int *queue = (int *)malloc(sizeof(int) * (size_t)n);
    int *seen = (int *)malloc(sizeof(int) * (size_t)n);
    int *done = (int *)calloc((size_t)n, sizeof(int));
    if (!level || !queue || !seen || !done) {
        free(xadj);
        free(adj);
        free(level);
        free(queue);
        free(seen);
        free(done);
        return spk_fail(SPIKE_ERR_MEMORY, "spike_rcm_permutation: host allocation failed");
    }
    for (int i = 0; i < n; i++) seen[i] = 0;
    int stamp = 0, out = 0;
    for (int s0 = 0; s0 < n; s0++) {
        if (done[s0]) continue;
        /* minimum-degree node of this component */
        int lb, ql;
        bfs_levels(s0, xadj, adj, level, queue, ++stamp, seen, &lb, &ql);
        int root = s0;
        for (int q = 0; q < ql; q++) {
            const int v = queue[q];
            if (xadj[v + 1] - xadj[v] < xadj[root + 1] - xadj[root]) root = v;
        }
        /* pseudo-peripheral node */
        int ecc = bfs_levels(root, xadj, adj, level, queue, ++stamp, seen, &lb, &ql);
        for (int it = 0; it < 16; it++) {
            int cand = queue[lb];
            for (int q = lb; q < ql; q++) {
                const int v = queue[q];
                if (xadj[v + 1] - xadj[v] < xadj[cand + 1] - xadj[cand]) cand = v;
            }
            const int e2 = bfs_levels(cand, xadj, adj, level, queue, ++stamp, seen, &lb, &ql);
            if (e2 <= ecc) break;
            ecc = e2;
            root = cand;
        }
        /* Cuthill-McKee from root: neighbours in increasing degree */
        int head = out, tail = out;
        perm[tail++] = root;
        done[root] = 1;
        while (head < tail) {
            const int v = perm[head++];
            const int first = tail;
            for (int t = xadj[v]; t < xadj[v + 1]; t++) {
                const int u = adj[t];
                if (done[u]) continue;
                done[u] = 1;
                int k = tail++;
                const int du = xadj[u + 1] - xadj[u];
                while (k > first && xadj[perm[k - 1] + 1] - xadj[perm[k - 1]] > du) {
                    perm[k] = perm[k - 1];
                    k--;
                }
                perm[k] = u;
            }
        }
        out = tail;
    }
    /* reverse */
    for (int i = 0, j = n - 1; i < j; i++, j--) {
        const int t = perm[i];
        perm[i] = perm[j];
        perm[j] = t;
    }
    free(xadj);
    free(adj);
    free(level);
    free(queue);
    free(seen);
    free(done);
    return spk_succeed();
}

Error_t spike_permute_csr(integer_t n, integer_t nnz, const integer_t *colind, const integer_t *rowptr,
                          const double *aij, const integer_t *perm, integer_t *out_colind, integer_t *out_rowptr,
                          double *out_aij)
{
    if (n < 0 || nnz < 0 || (n > 0 && (!colind || !rowptr || !aij || !perm || !out_colind || !out_rowptr || !out_aij)))
        return spk_fail(SPIKE_ERR_ARGUMENT, "spike_permute_csr: bad argument");
    int *inv = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!inv) return spk_fail(SPIKE_ERR_MEMORY, "spike_permute_csr: host allocation failed");
    for (int i = 0; i < n; i++) inv[i] = -1;
    for (int i = 0; i < n; i++) {
        if (perm[i] < 0 || perm[i] >= n || inv[perm[i]] >= 0) {
            free(inv);
            return spk_fail(SPIKE_ERR_ARGUMENT, "spike_permute_csr: perm is not a permutation");
        }
        inv[perm[i]] = i;
    }
    out_rowptr[0] = 0;
    for (int i = 0; i < n; i++) out_rowptr[i + 1] = out_rowptr[i] + (rowptr[perm[i] + 1] - rowptr[perm[i]]);
    for (int i = 0; i < n; i++) {
        const int src = perm[i], b = out_rowptr[i];
        int w = b;
        for (int t = rowptr[src]; t < rowptr[src + 1]; t++) {
            const int c = inv[colind[t]];
            const double v = aij[t];
            int k = w++;
            while (k > b && out_colind[k - 1] > c) { /* keep the row sorted */
                out_colind[k] = out_colind[k - 1];
                out_aij[k] = out_aij[k - 1];
                k--;
            }
            out_colind[k] = c;
            out_aij[k] = v;
        }
    }
    free(inv);
    return spk_succeed();
}

Error_t spike_permute_vector(integer_t flag, integer_t n, integer_t nrhs, const integer_t *perm, double *v)
{
    if (n < 0 || nrhs < 0 || (n > 0 && (!perm || !v))) return spk_fail(SPIKE_ERR_ARGUMENT, "spike_permute_vector: bad argument");
    double *work = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (!work) return spk_fail(SPIKE_ERR_MEMORY, "spike_permute_vector: host allocation failed");
    for (int h = 0; h < nrhs; h++) {
        double *col = v + (size_t)h * n;
        if (flag > 0)
            for (int i = 0; i < n; i++) work[i] = col[perm[i]];
        else
            for (int i = 0; i < n; i++) work[perm[i]] = col[i];
        memcpy(col, work, sizeof(double) * (size_t)n);
    }
    free(work);
    return spk_succeed();
}

Error_t spike_dsolve_reordered(spike_context_t ctx, integer_t n, integer_t nnz, integer_t nrhs,
                               const integer_t *colind, const integer_t *rowptr, const double *aij, double *x,
                               const double *b, integer_t *perm_out)
{
    const char *W = "spike_dsolve_reordered";
    if (n < 0 || nnz < 0 || nrhs < 0) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: n, nnz and nrhs must be >= 0", W);
    if (n == 0 || nrhs == 0) return spk_succeed();
    if (!colind || !rowptr || !aij || !x || !b) return spk_fail(SPIKE_ERR_ARGUMENT, "%s: NULL array", W);
    ctx = spk_get_ctx(ctx);
    if (!ctx) return SPIKE_ERROR;
    int *perm = (int *)malloc(sizeof(int) * (size_t)n);
    int *rp = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    int *ci = (int *)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    double *a = (double *)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    double *pb = (double *)malloc(sizeof(double) * (size_t)n * nrhs);
    Error_t rc = (perm && rp && ci && a && pb) ? SPIKE_SUCCESS : spk_fail(SPIKE_ERR_MEMORY, "%s: host allocation failed", W);
    if (rc == SPIKE_SUCCESS) rc = spike_rcm_permutation(n, nnz, colind, rowptr, perm);
    if (rc == SPIKE_SUCCESS) rc = spike_permute_csr(n, nnz, colind, rowptr, aij, perm, ci, rp, a);
    if (rc == SPIKE_SUCCESS) {
        memcpy(pb, b, sizeof(double) * (size_t)n * nrhs);
        rc = spike_permute_vector(1, n, nrhs, perm, pb); /* b(p) */
    }
    if (rc == SPIKE_SUCCESS) rc = spk_host_solve_ctx(ctx, SPK_D, W, n, nnz, nrhs, ci, rp, a, x, pb);
    if (rc == SPIKE_SUCCESS) rc = spike_permute_vector(0, n, nrhs, perm, x); /* x(p) = y */
    if (rc == SPIKE_SUCCESS && perm_out) memcpy(perm_out, perm, sizeof(int) * (size_t)n);
    free(perm);
    free(rp);
    free(ci);
    free(a);
    free(pb);
    return rc;
}
