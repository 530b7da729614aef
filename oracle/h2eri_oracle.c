/*
 * ORACLE - test infrastructure only. CPU restatement of the H2P-ERI hot path
 * used to check the GPU library (tests/, __graft_entry__.smoke) and as the
 * timed CPU baseline of bench.py. Never linked into the product.
 *
 * Parity pin: tests/test_oracle_pin.py runs the reference's own compiled
 * H2ERI_matvec / H2ERI_build_Coulomb / H2ERI_build_exchange (oracle/_ref,
 * built from the read-only reference sources where they exist) on the same
 * struct H2ERI and requires agreement to 1e-13; the J and K fixtures of the
 * reference test suite (tests/golden) pin the whole chain end to end.
 *
 * Functions follow:
 *   oracle_matvec          H2P-ERI src/H2ERI_matvec.c:882-957 (AOT branch)
 *     fwd                    src/H2ERI_matvec.c:93-175
 *     intermediate (B)       src/H2ERI_matvec.c:299-407
 *     bwd                    src/H2ERI_matvec.c:663-757
 *     dense (D)              src/H2ERI_matvec.c:572-660
 *     block bi-matvec        src/H2ERI_matvec.c:24-63, 225-264
 *   oracle_build_Coulomb   src/H2ERI_build_Coulomb.c:26-152
 *   oracle_build_exchange  src/H2ERI_build_exchange.c:193-1450
 * Thread-private partial outputs are summed at the end, as in the reference.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "h2eri_types.h"

/* y += A x, A row-major nrow x ncol with leading dimension lda; two rows
 * per pass over x */
static void gemv_n(int nrow, int ncol, const double *A, int lda, const double *x, double *y)
{
    int i = 0;
    for (; i + 1 < nrow; i += 2) {
        const double *a0 = A + (size_t)i * lda, *a1 = a0 + lda;
        double s0 = 0.0, s1 = 0.0;
        #pragma omp simd reduction(+ : s0, s1)
        for (int j = 0; j < ncol; j++) {
            s0 += a0[j] * x[j];
            s1 += a1[j] * x[j];
        }
        y[i] += s0;
        y[i + 1] += s1;
    }
    for (; i < nrow; i++) {
        const double *a = A + (size_t)i * lda;
        double s = 0.0;
        #pragma omp simd reduction(+ : s)
        for (int j = 0; j < ncol; j++) s += a[j] * x[j];
        y[i] += s;
    }
}

/* y += A^T x; two rows per pass over y */
static void gemv_t(int nrow, int ncol, const double *A, int lda, const double *x, double *y)
{
    int i = 0;
    for (; i + 1 < nrow; i += 2) {
        const double *a0 = A + (size_t)i * lda, *a1 = a0 + lda;
        const double x0 = x[i], x1 = x[i + 1];
        #pragma omp simd
        for (int j = 0; j < ncol; j++) y[j] += x0 * a0[j] + x1 * a1[j];
    }
    for (; i < nrow; i++) {
        const double *a = A + (size_t)i * lda;
        const double xi = x[i];
        #pragma omp simd
        for (int j = 0; j < ncol; j++) y[j] += a[j] * xi;
    }
}

/* out0 += A in0 and out1 += A^T in1 with one pass over A, two rows at a
 * time (the reference's CBLAS_BI_GEMV, src/H2ERI_matvec.c:24-63) */
static void bi_gemv(int nrow, int ncol, const double *A, int lda, const double *in0, const double *in1,
                    double *out0, double *out1)
{
    int i = 0;
    for (; i + 1 < nrow; i += 2) {
        const double *a0 = A + (size_t)i * lda, *a1 = a0 + lda;
        const double x0 = in1[i], x1 = in1[i + 1];
        double s0 = 0.0, s1 = 0.0;
        #pragma omp simd reduction(+ : s0, s1)
        for (int j = 0; j < ncol; j++) {
            s0 += a0[j] * in0[j];
            s1 += a1[j] * in0[j];
            out1[j] += x0 * a0[j] + x1 * a1[j];
        }
        out0[i] += s0;
        out0[i + 1] += s1;
    }
    for (; i < nrow; i++) {
        const double *a = A + (size_t)i * lda;
        const double x1 = in1[i];
        double s = 0.0;
        #pragma omp simd reduction(+ : s)
        for (int j = 0; j < ncol; j++) {
            s += a[j] * in0[j];
            out1[j] += a[j] * x1;
        }
        out0[i] += s;
    }
}

/* B or D block (dense, or low-rank U V with V^T stored): out0 += blk in0
 * (if out0) and out1 += blk^T in1 (if out1); tmp needs rank doubles */
static void blk_apply(const H2E_dense_mat_p blk, const double *in0, const double *in1, double *out0, double *out1,
                      double *tmp)
{
    if (blk->nrow == 0 || blk->ncol == 0) return;
    if (blk->ld > 0) {
        if (out0 && out1) bi_gemv(blk->nrow, blk->ncol, blk->data, blk->ld, in0, in1, out0, out1);
        else if (out0) gemv_n(blk->nrow, blk->ncol, blk->data, blk->ld, in0, out0);
        else if (out1) gemv_t(blk->nrow, blk->ncol, blk->data, blk->ld, in1, out1);
        return;
    }
    const int r = -blk->ld;
    const double *U = blk->data, *VT = U + (size_t)blk->nrow * r;
    if (out0) {
        memset(tmp, 0, sizeof(double) * r);
        gemv_t(blk->ncol, r, VT, r, in0, tmp);
        gemv_n(blk->nrow, r, U, r, tmp, out0);
    }
    if (out1) {
        memset(tmp, 0, sizeof(double) * r);
        gemv_t(blk->nrow, r, U, r, in1, tmp);
        gemv_n(blk->ncol, r, VT, r, tmp, out1);
    }
}

static int max_block_rank(H2ERI_p h)
{
    int m = 1;
    for (int i = 0; i < h->n_B; i++) if (h->c_B_blks[i]->ld < 0 && -h->c_B_blks[i]->ld > m) m = -h->c_B_blks[i]->ld;
    for (int i = 0; i < h->n_D; i++) if (h->c_D_blks[i]->ld < 0 && -h->c_D_blks[i]->ld > m) m = -h->c_D_blks[i]->ld;
    return m;
}

void oracle_matvec(H2ERI_p h, const double *x, double *y)
{
    const int n_node = h->n_node, krnl = h->krnl_mat_size, nt = omp_get_max_threads();
    const int nl = h->n_leaf_node;
    int *voff = (int *)malloc(sizeof(int) * (n_node + 1));
    voff[0] = 0;
    for (int i = 0; i < n_node; i++) voff[i + 1] = voff[i] + h->U[i]->ncol;
    const int rtot = voff[n_node];
    double *y0 = (double *)calloc((size_t)rtot + 1, sizeof(double));
    double *y1 = (double *)calloc((size_t)nt * rtot + 1, sizeof(double));
    double *yt = (double *)calloc((size_t)nt * krnl, sizeof(double));
    char *visited = (char *)calloc((size_t)n_node, 1);
    const int rmax = max_block_rank(h);
    double *tmp = (double *)malloc(sizeof(double) * (size_t)nt * rmax);

    /* upward sweep */
    for (int lv = h->max_level; lv >= h->min_adm_level; lv--) {
        const int *nodes = h->level_nodes + lv * nl;
        #pragma omp parallel for schedule(dynamic)
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = nodes[j];
            H2E_dense_mat_p U = h->U[node];
            if (U->ncol == 0) continue;
            double *out = y0 + voff[node];
            if (h->n_child[node] == 0) {
                gemv_t(U->nrow, U->ncol, U->data, U->ld, x + h->mat_cluster[2 * node], out);
            } else {
                int srow = 0;
                for (int k = 0; k < h->n_child[node]; k++) {
                    int c = h->children[node * h->max_child + k];
                    int nr = h->U[c]->ncol;
                    gemv_t(nr, U->ncol, U->data + (size_t)srow * U->ld, U->ld, y0 + voff[c], out);
                    srow += nr;
                }
            }
        }
    }
    /* intermediate multiplication */
    for (int i = 0; i < n_node; i++) visited[i] = (h->node_n_r_adm[i] > 0);
    #pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < h->n_r_adm_pair; i++) {
        int tid = omp_get_thread_num();
        double *y1t = y1 + (size_t)tid * rtot, *ytt = yt + (size_t)tid * krnl, *tp = tmp + (size_t)tid * rmax;
        int n0 = h->r_adm_pairs[2 * i], n1 = h->r_adm_pairs[2 * i + 1];
        int l0 = h->node_level[n0], l1 = h->node_level[n1];
        H2E_dense_mat_p B = h->c_B_blks[i];
        if (l0 == l1)
            blk_apply(B, y0 + voff[n1], y0 + voff[n0], y1t + voff[n0], y1t + voff[n1], tp);
        else if (l0 > l1) {
            int s1 = h->mat_cluster[2 * n1];
            blk_apply(B, x + s1, y0 + voff[n0], y1t + voff[n0], ytt + s1, tp);
        } else {
            int s0 = h->mat_cluster[2 * n0];
            blk_apply(B, y0 + voff[n1], x + s0, ytt + s0, y1t + voff[n1], tp);
        }
    }
    for (int t = 1; t < nt; t++)
        for (int k = 0; k < rtot; k++) y1[k] += y1[(size_t)t * rtot + k];
    /* downward sweep */
    memset(y, 0, sizeof(double) * krnl);
    for (int lv = h->min_adm_level; lv <= h->max_level; lv++) {
        const int *nodes = h->level_nodes + lv * nl;
        #pragma omp parallel for schedule(dynamic)
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = nodes[j];
            if (!visited[node]) continue;
            H2E_dense_mat_p U = h->U[node];
            double *t = (double *)calloc((size_t)U->nrow + 1, sizeof(double));
            gemv_n(U->nrow, U->ncol, U->data, U->ld, y1 + voff[node], t);
            if (h->n_child[node] == 0) {
                double *ys = y + h->mat_cluster[2 * node];
                for (int k = 0; k < U->nrow; k++) ys[k] += t[k];
            } else {
                int srow = 0;
                for (int k = 0; k < h->n_child[node]; k++) {
                    int c = h->children[node * h->max_child + k];
                    int nr = h->U[c]->ncol;
                    for (int l = 0; l < nr; l++) y1[voff[c] + l] += t[srow + l];
                    visited[c] = 1;
                    srow += nr;
                }
            }
            free(t);
        }
    }
    /* near field: diagonal blocks, then inadmissible pairs */
    #pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < h->n_D; i++) {
        int tid = omp_get_thread_num();
        double *ytt = yt + (size_t)tid * krnl, *tp = tmp + (size_t)tid * rmax;
        H2E_dense_mat_p Dm = h->c_D_blks[i];
        if (i < nl) {
            int s = h->mat_cluster[2 * h->height_nodes[i]];
            blk_apply(Dm, x + s, NULL, ytt + s, NULL, tp);
        } else {
            int k = i - nl, n0 = h->r_inadm_pairs[2 * k], n1 = h->r_inadm_pairs[2 * k + 1];
            int s0 = h->mat_cluster[2 * n0], s1 = h->mat_cluster[2 * n1];
            blk_apply(Dm, x + s1, x + s0, ytt + s0, ytt + s1, tp);
        }
    }
    #pragma omp parallel for schedule(static)
    for (int k = 0; k < krnl; k++) {
        double s = y[k];
        for (int t = 0; t < nt; t++) s += yt[(size_t)t * krnl + k];
        y[k] = s;
    }
    free(voff); free(y0); free(y1); free(yt); free(visited); free(tmp);
}

void oracle_build_Coulomb(H2ERI_p h, const double *den, double *J)
{
    const int nbf = h->num_bf, num_sp = h->num_sp, krnl = h->krnl_mat_size;
    double *x = (double *)malloc(sizeof(double) * (size_t)krnl);
    double *y = (double *)malloc(sizeof(double) * (size_t)krnl);
    #pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < num_sp; i++) {
        int M = h->sp_shell_idx[i], N = h->sp_shell_idx[i + num_sp];
        int srow = h->shell_bf_sidx[M], nrow = h->shell_bf_sidx[M + 1] - srow;
        int scol = h->shell_bf_sidx[N], ncol = h->shell_bf_sidx[N + 1] - scol;
        double c = (M == N) ? 1.0 : 2.0;
        for (int j = 0; j < ncol; j++)
            for (int k = 0; k < nrow; k++)
                x[h->sp_bfp_sidx[i] + j * nrow + k] = c * den[(size_t)(scol + j) * nbf + srow + k];
    }
    oracle_matvec(h, x, y);
    memset(J, 0, sizeof(double) * (size_t)nbf * nbf);
    #pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < num_sp; i++) {
        int M = h->sp_shell_idx[i], N = h->sp_shell_idx[i + num_sp];
        int srow = h->shell_bf_sidx[M], nrow = h->shell_bf_sidx[M + 1] - srow;
        int scol = h->shell_bf_sidx[N], ncol = h->shell_bf_sidx[N + 1] - scol;
        double c = (M == N) ? 0.5 : 1.0;
        for (int j = 0; j < ncol; j++)
            for (int k = 0; k < nrow; k++)
                J[(size_t)(scol + j) * nbf + srow + k] += c * y[h->sp_bfp_sidx[i] + j * nrow + k];
    }
    #pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < nbf; i++) {
        for (int j = 0; j < i; j++) {
            double v = J[(size_t)i * nbf + j] + J[(size_t)j * nbf + i];
            J[(size_t)i * nbf + j] = v;
            J[(size_t)j * nbf + i] = v;
        }
        J[(size_t)i * nbf + i] *= 2.0;
    }
    free(x);
    free(y);
}
