/*
 * ORACLE - test infrastructure only. CPU restatement of the H2P-ERI exchange
 * build (H2ERI_build_exchange) used to check the GPU library and as the timed
 * CPU baseline of the exchange benchmark. Never linked into the product.
 *
 * Algorithm (H2P-ERI src/H2ERI_build_exchange.c:1356-1450): for every pair of
 * shells (N, Q) one partial H2 product
 *     Y[(m,n)][(q,n')] = sum_(p,q') A[(m,n),(p,q')] X[(p,q')][(q,n')]
 * is formed whose input columns are the N_nbf * Q_nbf pairs (q, n') and whose
 * input rows are the basis-function pairs of the screened shell pairs (P, Q)
 * with P in plist[Q] and D[N, P] significant (dlist, :771-838), holding
 * X[(p,q)][(q,n)] = D[p][n] (:590-650). Only rows of the shell pairs (M, N),
 * M in plist[N], are produced (:238-350) and K[m][q] += sum_n Y[(m,n)][(q,n)]
 * (:723-768). The partial product walks the smallest subtrees that cover the
 * input rows (column side) and output rows (row side) (:193-245):
 *   forward   y0 = U^T x over the column subtree           (:1101-1155)
 *   coupling  B blocks between row-side and column-side nodes, in the three
 *             level cases of the matvec                    (:1160-1250)
 *   backward  y1 pushed down the row subtree               (:1253-1305)
 *   near      D blocks between row-side and column-side leaves (:1307-1350)
 * Levels outside [col/row subtree depth, min_adm_level] only hold zeros in
 * the reference (:1080-1099); here they are simply not visited. Within a
 * leaf only the selected rows are touched, like the reference's nnz row
 * lists. Shells are processed in parallel over N with thread-private K
 * copies summed at the end (the reference adds into K with atomics).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "h2eri_types.h"

/* Significance test of a density block (src/H2ERI_build_exchange.c:784-806) */
#define ORACLE_K_DTOL 1e-10

/* Beff = blk or blk^T (trans); out[i][:] += sum_j Beff[rows[i]][cols[j]] in[j][:]
 * (rows / cols NULL = all), vectors nvec wide. tmp: rank * nvec doubles. */
static void blk_sub_mm(const H2E_dense_mat_p blk, int trans, int nr, const int *rows, int nc, const int *cols,
                       const double *in, double *out, int nvec, double *tmp)
{
    if (blk->nrow == 0 || blk->ncol == 0 || nr == 0 || nc == 0) return;
    if (blk->ld > 0) {
        for (int i = 0; i < nr; i++) {
            int ri = rows ? rows[i] : i;
            double *o = out + (size_t)i * nvec;
            for (int j = 0; j < nc; j++) {
                int cj = cols ? cols[j] : j;
                double a = trans ? blk->data[(size_t)cj * blk->ld + ri] : blk->data[(size_t)ri * blk->ld + cj];
                const double *x = in + (size_t)j * nvec;
                for (int v = 0; v < nvec; v++) o[v] += a * x[v];
            }
        }
        return;
    }
    /* low rank: blk = Ub * VT^T, Ub nrow x r, VT ncol x r (src/H2ERI_build_exchange.c:911-967) */
    const int r = -blk->ld;
    const double *Ub = blk->data, *VT = Ub + (size_t)blk->nrow * r;
    const double *L = trans ? VT : Ub;   /* Beff = L * R^T */
    const double *R = trans ? Ub : VT;
    memset(tmp, 0, sizeof(double) * (size_t)r * nvec);
    for (int j = 0; j < nc; j++) {
        const double *rr = R + (size_t)(cols ? cols[j] : j) * r;
        const double *x = in + (size_t)j * nvec;
        for (int k = 0; k < r; k++) {
            double a = rr[k];
            for (int v = 0; v < nvec; v++) tmp[(size_t)k * nvec + v] += a * x[v];
        }
    }
    for (int i = 0; i < nr; i++) {
        const double *lr = L + (size_t)(rows ? rows[i] : i) * r;
        double *o = out + (size_t)i * nvec;
        for (int k = 0; k < r; k++) {
            double a = lr[k];
            const double *t = tmp + (size_t)k * nvec;
            for (int v = 0; v < nvec; v++) o[v] += a * t[v];
        }
    }
}

/* Block index of the (n0, n1) pair in a node-pair CSR map; < 0 = stored as (n1, n0). */
static int csr_get(const int *rowptr, const int *colidx, const int *val, int r, int c)
{
    for (int k = rowptr[r]; k < rowptr[r + 1]; k++)
        if (colidx[k] == c) return val[k];
    return 0;
}

/* Rows of a shell pair (X, Y) as seen from the outer shell Y with partner X:
 * matrix row of (x, y) for x in X, y in Y. The pair is stored once, as
 * (min, max), with basis-function pairs second-major (src/H2ERI_build_exchange.c
 * :303-325 for the row side, :420-445 for the column side). */
static int pair_row(const H2ERI_p h, int pair, int X, int Y, int xl, int yl)
{
    int nX = h->shell_bf_sidx[X + 1] - h->shell_bf_sidx[X];
    int nY = h->shell_bf_sidx[Y + 1] - h->shell_bf_sidx[Y];
    return h->sp_bfp_sidx[pair] + ((X <= Y) ? yl * nX + xl : xl * nY + yl);
}

typedef struct {
    int *cnt, *off;        /* per node: number / offset of selected leaf rows */
    int *rows;             /* local row in the leaf                          */
    int *a, *b;            /* row side: m (global bf), n (local in N); column side: p (global), q (local in Q) */
    int *flag;             /* node in the covering subtree                   */
    int total;
} side_sel;

static void side_alloc(side_sel *s, int n_node, int cap)
{
    s->cnt = (int *)calloc((size_t)n_node, sizeof(int));
    s->off = (int *)calloc((size_t)n_node + 1, sizeof(int));
    s->rows = (int *)malloc(sizeof(int) * (size_t)(cap + 1));
    s->a = (int *)malloc(sizeof(int) * (size_t)(cap + 1));
    s->b = (int *)malloc(sizeof(int) * (size_t)(cap + 1));
    s->flag = (int *)calloc((size_t)n_node, sizeof(int));
    s->total = 0;
}

static void side_free(side_sel *s)
{
    free(s->cnt); free(s->off); free(s->rows); free(s->a); free(s->b); free(s->flag);
}

/* Fill a side selection from a list of (matrix row, a, b) triples: bucket by
 * leaf, then mark the covering subtree (src/H2ERI_build_exchange.c:193-245). */
static void side_build(const H2ERI_p h, const int *row_leaf, side_sel *s, int n, const int *r, const int *a,
                       const int *b)
{
    const int n_node = h->n_node;
    memset(s->cnt, 0, sizeof(int) * (size_t)n_node);
    memset(s->flag, 0, sizeof(int) * (size_t)n_node);
    for (int i = 0; i < n; i++) s->cnt[row_leaf[r[i]]]++;
    s->off[0] = 0;
    for (int i = 0; i < n_node; i++) s->off[i + 1] = s->off[i] + s->cnt[i];
    memset(s->cnt, 0, sizeof(int) * (size_t)n_node);
    for (int i = 0; i < n; i++) {
        int leaf = row_leaf[r[i]];
        int k = s->off[leaf] + s->cnt[leaf]++;
        s->rows[k] = r[i] - h->mat_cluster[2 * leaf];
        s->a[k] = a[i];
        s->b[k] = b[i];
    }
    s->total = n;
    for (int i = 0; i < n_node; i++) {
        if (s->cnt[i] == 0) continue;
        for (int node = i; node >= 0 && !s->flag[node]; node = h->parent[node]) s->flag[node] = 1;
    }
}

static int max_rank_any(const H2ERI_p h)
{
    int m = 1;
    for (int i = 0; i < h->n_node; i++) if (h->U[i]->ncol > m) m = h->U[i]->ncol;
    for (int i = 0; i < h->n_B; i++) if (h->c_B_blks[i]->ld < 0 && -h->c_B_blks[i]->ld > m) m = -h->c_B_blks[i]->ld;
    for (int i = 0; i < h->n_D; i++) if (h->c_D_blks[i]->ld < 0 && -h->c_D_blks[i]->ld > m) m = -h->c_D_blks[i]->ld;
    return m;
}

/* One (N, Q) partial product (src/H2ERI_build_exchange.c:1021-1353) on the
 * prepared row side rs (rows of the pairs with N) and column side cs. x: the
 * column side's compact input, yr: the row side's compact output (zeroed),
 * y0 / y1: per-node skeleton coefficients (voff offsets, nvec wide). */
static void partial_product(const H2ERI_p h, const side_sel *rs, const side_sel *cs, const int *voff, int nvec,
                            const double *x, double *yr, double *y0, double *y1, double *tmp)
{
    const int nl = h->n_leaf_node;
    for (int i = 0; i < h->n_node; i++) {
        if (cs->flag[i]) memset(y0 + (size_t)voff[i] * nvec, 0, sizeof(double) * (size_t)h->U[i]->ncol * nvec);
        if (rs->flag[i]) memset(y1 + (size_t)voff[i] * nvec, 0, sizeof(double) * (size_t)h->U[i]->ncol * nvec);
    }
    /* forward transform over the column subtree (:1101-1155) */
    for (int lv = h->max_level; lv >= h->min_adm_level; lv--) {
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = h->level_nodes[lv * nl + j];
            if (!cs->flag[node]) continue;
            H2E_dense_mat_p U = h->U[node];
            const int rk = U->ncol;
            double *out = y0 + (size_t)voff[node] * nvec;
            if (h->n_child[node] == 0) {
                for (int k = cs->off[node]; k < cs->off[node + 1]; k++) {
                    const double *u = U->data + (size_t)cs->rows[k] * U->ld;
                    const double *xv = x + (size_t)k * nvec;
                    for (int t = 0; t < rk; t++)
                        for (int v = 0; v < nvec; v++) out[(size_t)t * nvec + v] += u[t] * xv[v];
                }
            } else {
                int srow = 0;
                for (int c = 0; c < h->n_child[node]; c++) {
                    int ch = h->children[node * h->max_child + c];
                    int rc = h->U[ch]->ncol;
                    if (cs->flag[ch]) {
                        const double *yc = y0 + (size_t)voff[ch] * nvec;
                        for (int t = 0; t < rc; t++) {
                            const double *u = U->data + (size_t)(srow + t) * U->ld;
                            for (int s = 0; s < rk; s++)
                                for (int v = 0; v < nvec; v++) out[(size_t)s * nvec + v] += u[s] * yc[(size_t)t * nvec + v];
                        }
                    }
                    srow += rc;
                }
            }
        }
    }
    /* coupling blocks (:1160-1250) */
    for (int n0 = 0; n0 < h->n_node; n0++) {
        if (!rs->flag[n0]) continue;
        for (int k = h->node_adm_pairs_sidx[n0]; k < h->node_adm_pairs_sidx[n0 + 1]; k++) {
            int n1 = h->node_adm_pairs[k];
            if (!cs->flag[n1]) continue;
            int pi = csr_get(h->B_p2i_rowptr, h->B_p2i_colidx, h->B_p2i_val, n0, n1);
            if (pi == 0) abort();
            int trans = pi < 0;
            H2E_dense_mat_p B = h->c_B_blks[(trans ? -pi : pi) - 1];
            int l0 = h->node_level[n0], l1 = h->node_level[n1];
            int r0 = h->U[n0]->ncol, r1 = h->U[n1]->ncol;
            if (l0 == l1) {
                blk_sub_mm(B, trans, r0, NULL, r1, NULL, y0 + (size_t)voff[n1] * nvec, y1 + (size_t)voff[n0] * nvec,
                           nvec, tmp);
            } else if (l0 > l1) {
                int c0 = cs->off[n1], nc = cs->off[n1 + 1] - c0;
                blk_sub_mm(B, trans, r0, NULL, nc, cs->rows + c0, x + (size_t)c0 * nvec, y1 + (size_t)voff[n0] * nvec,
                           nvec, tmp);
            } else {
                int o0 = rs->off[n0], nr = rs->off[n0 + 1] - o0;
                blk_sub_mm(B, trans, nr, rs->rows + o0, r1, NULL, y0 + (size_t)voff[n1] * nvec, yr + (size_t)o0 * nvec,
                           nvec, tmp);
            }
        }
    }
    /* backward transform over the row subtree (:1253-1305) */
    for (int lv = h->min_adm_level; lv <= h->max_level; lv++) {
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = h->level_nodes[lv * nl + j];
            if (!rs->flag[node]) continue;
            H2E_dense_mat_p U = h->U[node];
            const int rk = U->ncol;
            const double *in = y1 + (size_t)voff[node] * nvec;
            if (h->n_child[node] == 0) {
                for (int k = rs->off[node]; k < rs->off[node + 1]; k++) {
                    const double *u = U->data + (size_t)rs->rows[k] * U->ld;
                    double *o = yr + (size_t)k * nvec;
                    for (int s = 0; s < rk; s++)
                        for (int v = 0; v < nvec; v++) o[v] += u[s] * in[(size_t)s * nvec + v];
                }
            } else {
                int srow = 0;
                for (int c = 0; c < h->n_child[node]; c++) {
                    int ch = h->children[node * h->max_child + c];
                    int rc = h->U[ch]->ncol;
                    if (rs->flag[ch]) {
                        double *yc = y1 + (size_t)voff[ch] * nvec;
                        for (int t = 0; t < rc; t++) {
                            const double *u = U->data + (size_t)(srow + t) * U->ld;
                            for (int s = 0; s < rk; s++)
                                for (int v = 0; v < nvec; v++) yc[(size_t)t * nvec + v] += u[s] * in[(size_t)s * nvec + v];
                        }
                    }
                    srow += rc;
                }
            }
        }
    }
    /* near-field blocks between selected leaves (:1307-1350) */
    for (int n0 = 0; n0 < h->n_node; n0++) {
        int o0 = rs->off[n0], nr = rs->off[n0 + 1] - o0;
        if (nr == 0) continue;
        for (int k = h->node_inadm_pairs_sidx[n0]; k < h->node_inadm_pairs_sidx[n0 + 1]; k++) {
            int n1 = h->node_inadm_pairs[k];
            int c0 = cs->off[n1], nc = cs->off[n1 + 1] - c0;
            if (nc == 0) continue;
            int pi = csr_get(h->D_p2i_rowptr, h->D_p2i_colidx, h->D_p2i_val, n0, n1);
            if (pi == 0) abort();
            int trans = pi < 0;
            H2E_dense_mat_p Dm = h->c_D_blks[(trans ? -pi : pi) - 1];
            blk_sub_mm(Dm, trans, nr, rs->rows + o0, nc, cs->rows + c0, x + (size_t)c0 * nvec, yr + (size_t)o0 * nvec,
                       nvec, tmp);
        }
    }
}

/* The contributions of the outer shells N in Nlist[0..nN) to K (the
 * reference's N loop, src/H2ERI_build_exchange.c:1386-1425); all shells give
 * the full K. */
void oracle_build_exchange_shells(H2ERI_p h, const double *den, double *K, const int *Nlist, int n_list)
{
    const int nbf = h->num_bf, nsh = h->nshell, n_node = h->n_node, krnl = h->krnl_mat_size;
    const int *sb = h->shell_bf_sidx;
    const int nt = omp_get_max_threads();
    const int mnbf = h->max_shell_nbf, nvmax = mnbf * mnbf;

    /* dlist: shell blocks D[N, P] with an element above the threshold (:771-838) */
    char *sig = (char *)calloc((size_t)nsh * nsh, 1);
    #pragma omp parallel for schedule(dynamic)
    for (int N = 0; N < nsh; N++)
        for (int P = 0; P < nsh; P++) {
            int hit = 0;
            for (int i = sb[N]; i < sb[N + 1] && !hit; i++)
                for (int j = sb[P]; j < sb[P + 1]; j++)
                    if (fabs(den[(size_t)i * nbf + j]) > ORACLE_K_DTOL) { hit = 1; break; }
            sig[(size_t)N * nsh + P] = (char)hit;
        }

    /* matrix row -> leaf node */
    int *row_leaf = (int *)malloc(sizeof(int) * (size_t)(krnl + 1));
    for (int i = 0; i < h->n_leaf_node; i++) {
        int node = h->height_nodes[i];
        for (int r = h->mat_cluster[2 * node]; r <= h->mat_cluster[2 * node + 1]; r++) row_leaf[r] = node;
    }
    int *voff = (int *)malloc(sizeof(int) * (size_t)(n_node + 1));
    voff[0] = 0;
    for (int i = 0; i < n_node; i++) voff[i + 1] = voff[i] + h->U[i]->ncol;
    int max_np = 0;
    for (int s = 0; s < nsh; s++) {
        int cnt = 0;
        for (int k = h->plist_sidx[s]; k < h->plist_sidx[s + 1]; k++) cnt += sb[h->plist[k] + 1] - sb[h->plist[k]];
        if (cnt > max_np) max_np = cnt;
    }
    const int cap = max_np * mnbf;   /* rows of all pairs with one shell */
    const int rmax = max_rank_any(h);
    double *Kt = (double *)calloc((size_t)nt * nbf * nbf, sizeof(double));

    #pragma omp parallel num_threads(nt)
    {
        const int tid = omp_get_thread_num();
        double *Kp = Kt + (size_t)tid * nbf * nbf;
        side_sel rs, cs;
        side_alloc(&rs, n_node, cap);
        side_alloc(&cs, n_node, cap);
        int *lr = (int *)malloc(sizeof(int) * (size_t)(cap + 1));
        int *la = (int *)malloc(sizeof(int) * (size_t)(cap + 1));
        int *lb = (int *)malloc(sizeof(int) * (size_t)(cap + 1));
        double *x = (double *)malloc(sizeof(double) * ((size_t)cap * nvmax + 1));
        double *yr = (double *)malloc(sizeof(double) * ((size_t)cap * nvmax + 1));
        double *y0 = (double *)malloc(sizeof(double) * ((size_t)voff[n_node] * nvmax + 1));
        double *y1 = (double *)malloc(sizeof(double) * ((size_t)voff[n_node] * nvmax + 1));
        double *tmp = (double *)malloc(sizeof(double) * ((size_t)rmax * nvmax + 1));

        #pragma omp for schedule(dynamic)
        for (int iN = 0; iN < n_list; iN++) {
            const int N = Nlist[iN];
            const int nN = sb[N + 1] - sb[N];
            /* row side: (m, n) for M in plist[N] (:248-350) */
            int n = 0;
            for (int k = h->plist_sidx[N]; k < h->plist_sidx[N + 1]; k++) {
                int M = h->plist[k], pair = h->plist_idx[k], nM = sb[M + 1] - sb[M];
                for (int nl = 0; nl < nN; nl++)
                    for (int ml = 0; ml < nM; ml++) {
                        lr[n] = pair_row(h, pair, M, N, ml, nl);
                        la[n] = sb[M] + ml;
                        lb[n] = nl;
                        n++;
                    }
            }
            side_build(h, row_leaf, &rs, n, lr, la, lb);

            for (int Q = 0; Q < nsh; Q++) {
                const int nQ = sb[Q + 1] - sb[Q], nvec = nN * nQ;
                /* column side: (p, q) for P in plist[Q] with D[N, P] significant (:405-445) */
                int c = 0;
                for (int k = h->plist_sidx[Q]; k < h->plist_sidx[Q + 1]; k++) {
                    int P = h->plist[k], pair = h->plist_idx[k], nP = sb[P + 1] - sb[P];
                    if (!sig[(size_t)N * nsh + P]) continue;
                    for (int ql = 0; ql < nQ; ql++)
                        for (int pl = 0; pl < nP; pl++) {
                            lr[c] = pair_row(h, pair, P, Q, pl, ql);
                            la[c] = sb[P] + pl;
                            lb[c] = ql;
                            c++;
                        }
                }
                if (c == 0) continue;
                side_build(h, row_leaf, &cs, c, lr, la, lb);
                /* X[(p,q)][(q',n)] = delta(q,q') D[p][n] (:590-650) */
                for (int k = 0; k < c; k++) {
                    double *xr = x + (size_t)k * nvec;
                    memset(xr, 0, sizeof(double) * (size_t)nvec);
                    const double *dr = den + (size_t)cs.a[k] * nbf + sb[N];
                    for (int nl = 0; nl < nN; nl++) xr[cs.b[k] * nN + nl] = dr[nl];
                }
                memset(yr, 0, sizeof(double) * (size_t)rs.total * nvec);
                partial_product(h, &rs, &cs, voff, nvec, x, yr, y0, y1, tmp);
                /* K[m][q] += sum_n Y[(m,n)][(q,n)] (:723-768) */
                for (int k = 0; k < rs.total; k++) {
                    const double *yv = yr + (size_t)k * nvec;
                    double *kr = Kp + (size_t)rs.a[k] * nbf + sb[Q];
                    for (int ql = 0; ql < nQ; ql++) kr[ql] += yv[ql * nN + rs.b[k]];
                }
            }
        }
        side_free(&rs); side_free(&cs);
        free(lr); free(la); free(lb); free(x); free(yr); free(y0); free(y1); free(tmp);
    }
    #pragma omp parallel for schedule(static)
    for (size_t i = 0; i < (size_t)nbf * nbf; i++) {
        double s = 0.0;
        for (int t = 0; t < nt; t++) s += Kt[(size_t)t * nbf * nbf + i];
        K[i] = s;
    }
    free(Kt); free(voff); free(row_leaf); free(sig);
}

/* K = exchange matrix of the symmetric density den (both num_bf^2, row-major);
 * src/H2ERI_build_exchange.c:1356-1450 */
void oracle_build_exchange(H2ERI_p h, const double *den, double *K)
{
    int *all = (int *)malloc(sizeof(int) * (size_t)(h->nshell + 1));
    for (int i = 0; i < h->nshell; i++) all[i] = i;
    oracle_build_exchange_shells(h, den, K, all, h->nshell);
    free(all);
}
