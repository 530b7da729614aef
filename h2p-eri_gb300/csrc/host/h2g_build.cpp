/*
 * Per-geometry H2 construction on the host (runs once before upload):
 * nested bases U from proxy points and far-field sketches, coupling blocks B,
 * near-field blocks D, and their interpolative-decomposition compression.
 * Restates H2P-ERI src/H2ERI_build_H2.c and src/H2E_ID_compress.c; the random
 * sketches use a deterministic per-node generator instead of libc rand(), so
 * the result is reproducible run to run (the reference's is not: rand() is
 * called from OpenMP threads, src/H2ERI_utils.c:68,77).
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>
#include <omp.h>

#include "h2g_eri.h"
#include "h2g_host.h"
#include "h2eri_gb300.h"

namespace h2g {

/* ---------------------------------------------------------------------- */
/* Pivoted QR and interpolative decomposition                              */
/* ---------------------------------------------------------------------- */

/* Two-wide double vectors (GCC vector extension, no instruction-set header):
 * element-wise IEEE arithmetic, so every host computes the same bits. */
typedef double v2d __attribute__((vector_size(16)));

static inline v2d ld2(const double *p) { v2d v; std::memcpy(&v, p, sizeof v); return v; }
static inline void st2(double *p, v2d v) { std::memcpy(p, &v, sizeof v); }
static inline v2d bc2(double x) { v2d v = {x, x}; return v; }
static inline double hsum(v2d a, v2d b) { return (a[0] + b[0]) + (a[1] + b[1]); }

/* a . b over n elements: four partial sums (elements i mod 4), combined in a
 * fixed order, then the remainder */
static double dot(const double *a, const double *b, int n)
{
    v2d s0 = bc2(0.0), s1 = bc2(0.0);
    int i = 0;
    for (; i + 4 <= n; i += 4) {
        s0 += ld2(a + i) * ld2(b + i);
        s1 += ld2(a + i + 2) * ld2(b + i + 2);
    }
    double r = hsum(s0, s1);
    for (; i < n; i++) r += a[i] * b[i];
    return r;
}

/* out[q] = dot(c[q], x, n) for four columns, the same sums as dot() */
static void dot4(const double *const *c, const double *x, int n, double *out)
{
    const double *c0 = c[0], *c1 = c[1], *c2 = c[2], *c3 = c[3];
    v2d a0 = bc2(0.0), b0 = a0, a1 = a0, b1 = a0, a2 = a0, b2 = a0, a3 = a0, b3 = a0;
    int i = 0;
    for (; i + 4 <= n; i += 4) {
        const v2d xa = ld2(x + i), xb = ld2(x + i + 2);
        a0 += ld2(c0 + i) * xa; b0 += ld2(c0 + i + 2) * xb;
        a1 += ld2(c1 + i) * xa; b1 += ld2(c1 + i + 2) * xb;
        a2 += ld2(c2 + i) * xa; b2 += ld2(c2 + i + 2) * xb;
        a3 += ld2(c3 + i) * xa; b3 += ld2(c3 + i + 2) * xb;
    }
    double r0 = hsum(a0, b0), r1 = hsum(a1, b1), r2 = hsum(a2, b2), r3 = hsum(a3, b3);
    for (; i < n; i++) {
        r0 += c0[i] * x[i];
        r1 += c1[i] * x[i];
        r2 += c2[i] * x[i];
        r3 += c3[i] * x[i];
    }
    out[0] = r0; out[1] = r1; out[2] = r2; out[3] = r3;
}

/* c[lo:m) -= sum_t v_t[lo:m) f[t], t = 0..k-1, with v_t = v + t * ld; every
 * element subtracts its k products in the order of t. Two columns at once
 * (c2/f2 non-null) share the loads of v. */
static void apply_block(double *c, const double *f, double *c2, const double *f2,
                        const double *v, int ld, int k, int lo, int m)
{
    int i = lo;
    if (c2) {
        for (; i + 4 <= m; i += 4) {
            v2d a = ld2(c + i), b = ld2(c + i + 2), a2 = ld2(c2 + i), b2 = ld2(c2 + i + 2);
            for (int t = 0; t < k; t++) {
                const double *vt = v + (size_t)t * ld + i;
                const v2d va = ld2(vt), vb = ld2(vt + 2), ft = bc2(f[t]), ft2 = bc2(f2[t]);
                a -= va * ft;  b -= vb * ft;
                a2 -= va * ft2; b2 -= vb * ft2;
            }
            st2(c + i, a); st2(c + i + 2, b);
            st2(c2 + i, a2); st2(c2 + i + 2, b2);
        }
    } else {
        for (; i + 4 <= m; i += 4) {
            v2d a = ld2(c + i), b = ld2(c + i + 2);
            for (int t = 0; t < k; t++) {
                const double *vt = v + (size_t)t * ld + i;
                const v2d ft = bc2(f[t]);
                a -= ld2(vt) * ft;
                b -= ld2(vt + 2) * ft;
            }
            st2(c + i, a); st2(c + i + 2, b);
        }
    }
    for (; i < m; i++) {
        double s = c[i], s2 = c2 ? c2[i] : 0.0;
        for (int t = 0; t < k; t++) {
            const double vt = v[(size_t)t * ld + i];
            s -= vt * f[t];
            if (c2) s2 -= vt * f2[t];
        }
        c[i] = s;
        if (c2) c2[i] = s2;
    }
}

/* Reflectors t = t0..t1-1 applied in order to column c (rows t..m): v_t is
 * column t of A below row t with a unit leading entry (the stored diagonal,
 * R's, is not read), tau[t - toff] its factor. */
static void apply_reflectors(double *c, const double *A, int ld, int m, const double *tau, int toff, int t0,
                             int t1)
{
    for (int t = t0; t < t1; t++) {
        const double *v = A + (size_t)t * ld;
        const double w = tau[t - toff] * (c[t] + dot(v + t + 1, c + t + 1, m - t - 1));
        c[t] -= w;
        const v2d wv = bc2(w);
        int i = t + 1;
        for (; i + 2 <= m; i += 2) st2(c + i, ld2(c + i) - wv * ld2(v + i));
        for (; i < m; i++) c[i] -= w * v[i];
    }
}

/* Householder QR with column pivoting on a column-major m x n matrix A
 * (leading dimension ld), stopping when the largest remaining column norm
 * drops below rel_tol times the largest initial column norm, with the
 * reference's pivot rule, reflectors and stopping test
 * (H2P-ERI src/H2E_ID_compress.c:51-184). Returns the rank r; rows 0..r-1
 * of A then hold R11 and R12 and p the column permutation.
 *
 * Blocked as in LAPACK's xLAQPS: within a block of up to kQrBlock
 * reflectors only the pivot column and the pivot row are brought up to date,
 * the other columns' pending updates are kept in F (current column j =
 * stored column j - V F(j, :)^T), and the trailing matrix is updated once
 * per block, so each step reads the trailing matrix once instead of reading
 * and writing it. Partial column norms are downdated from the pivot row;
 * where the downdate has lost its accuracy (LAPACK's test, in place of the
 * reference's absolute threshold 1e-10 on the squared norm) the column is
 * brought up to date and its norm taken again.
 *
 * A column whose norm is below the stop norm (the reference sets its norm to
 * zero: it is never a pivot again) leaves the per-step work: it is brought up
 * to date once and receives each block's reflectors in order when the block
 * ends, which still gives its R12 entries. The pivots and the live columns
 * are computed exactly as without this. On the largest U-construction
 * matrices the share of trailing columns below the stop norm grows from about
 * 10 % at the first step to over 90 % near the rank. */
static int pivoted_qr(double *A, int m, int n, int ld, double rel_tol, int *p)
{
    constexpr int kQrBlock = 32;
    const double kDowndateTol = 1.4901161193847656e-08;   /* sqrt(2^-52) */
    const int kmax = std::min(m, n);
    std::vector<double> vn1(n), vn2(n), F((size_t)n * kQrBlock, 0.0), aux(kQrBlock), tau(kQrBlock);
    /* done[j] >= 0: column j is below the stop norm and current through reflector done[j] - 1 */
    std::vector<int> done(n, -1), live;
    live.reserve(n);
    double norm0 = 0.0;
    for (int j = 0; j < n; j++) {
        p[j] = j;
        const double *c = A + (size_t)j * ld;
        vn1[j] = vn2[j] = std::sqrt(dot(c, c, m));
        norm0 = std::max(norm0, vn1[j]);
    }
    if (!(norm0 > 0.0)) return 0;   /* a zero matrix has rank 0 (no zero pivots) */
    const double stop = std::max(std::sqrt((double)m) * 1e-15, rel_tol) * norm0;
    for (int j = 0; j < n; j++)
        if (vn1[j] < stop) { vn1[j] = 0.0; done[j] = 0; }
    int off = 0;
    while (off < kmax) {
        const int nb = std::min(kQrBlock, kmax - off);
        const double *V = A + (size_t)off * ld;
        int k = 0;
        for (; k < nb; k++) {
            const int rk = off + k;
            int pvt = rk;
            for (int j = rk + 1; j < n; j++)
                if (vn1[j] > vn1[pvt]) pvt = j;
            if (vn1[pvt] < stop) break;
            if (pvt != rk) {
                double *a = A + (size_t)rk * ld, *b = A + (size_t)pvt * ld;
                for (int i = 0; i < m; i++) std::swap(a[i], b[i]);
                for (int t = 0; t < k; t++) std::swap(F[(size_t)rk * kQrBlock + t], F[(size_t)pvt * kQrBlock + t]);
                std::swap(p[rk], p[pvt]);
                std::swap(vn1[rk], vn1[pvt]);
                std::swap(vn2[rk], vn2[pvt]);
                std::swap(done[rk], done[pvt]);
            }
            live.clear();
            for (int j = rk + 1; j < n; j++)
                if (done[j] < 0) live.push_back(j);
            const int nl = (int)live.size();
            double *x = A + (size_t)rk * ld;
            /* the pivot column, up to date below its pivot row */
            apply_block(x, &F[(size_t)rk * kQrBlock], nullptr, nullptr, V, ld, k, rk, m);
            /* reflector I - tau v v^T with v = (1, x[rk+1:m) / (alpha - beta)) */
            const double alpha = x[rk];
            const double xn = dot(x + rk + 1, x + rk + 1, m - rk - 1);
            double tk = 0.0, beta = alpha;
            if (xn > 0.0) {
                beta = -std::copysign(std::sqrt(alpha * alpha + xn), alpha);
                tk = (beta - alpha) / beta;
                const double sc = 1.0 / (alpha - beta);
                for (int i = rk + 1; i < m; i++) x[i] *= sc;
            }
            tau[k] = tk;
            x[rk] = 1.0;
            /* F(j, k) = tau (A(rk:m, j)^T v) + F(j, 0:k) aux, aux = -tau V(rk:m, 0:k)^T v */
            int q = 0;
            double d4[4];
            for (; q + 4 <= nl; q += 4) {
                const double *cs[4];
                for (int u = 0; u < 4; u++) cs[u] = A + (size_t)live[q + u] * ld + rk;
                dot4(cs, x + rk, m - rk, d4);
                for (int u = 0; u < 4; u++) F[(size_t)live[q + u] * kQrBlock + k] = tk * d4[u];
            }
            for (; q < nl; q++) F[(size_t)live[q] * kQrBlock + k] = tk * dot(A + (size_t)live[q] * ld + rk, x + rk, m - rk);
            if (k > 0) {
                for (int t = 0; t < k; t++) aux[t] = -tk * dot(V + (size_t)t * ld + rk, x + rk, m - rk);
                for (int j : live) {
                    double *f = &F[(size_t)j * kQrBlock];
                    double s = 0.0;
                    for (int t = 0; t < k; t++) s += f[t] * aux[t];
                    f[k] += s;
                }
            }
            /* the pivot row: A(rk, j) -= A(rk, off:rk+1) F(j, 0:k+1)^T */
            for (int j : live) {
                const double *f = &F[(size_t)j * kQrBlock];
                double s = 0.0;
                for (int t = 0; t <= k; t++) s += V[(size_t)t * ld + rk] * f[t];
                A[(size_t)j * ld + rk] -= s;
            }
            x[rk] = beta;
            /* downdate the remaining column norms */
            for (int j : live) {
                double *c = A + (size_t)j * ld;
                double *f = &F[(size_t)j * kQrBlock];
                if (vn1[j] < stop) {   /* below the stop norm from now on */
                    apply_block(c, f, nullptr, nullptr, V, ld, k + 1, rk + 1, m);
                    std::fill(f, f + k + 1, 0.0);
                    vn1[j] = 0.0;
                    done[j] = rk + 1;
                    continue;
                }
                const double qn = std::fabs(c[rk]) / vn1[j];
                const double t = std::max(0.0, (1.0 + qn) * (1.0 - qn));
                const double r = vn1[j] / vn2[j];
                if (t * r * r > kDowndateTol) {
                    vn1[j] *= std::sqrt(t);
                    continue;
                }
                apply_block(c, f, nullptr, nullptr, V, ld, k + 1, rk + 1, m);
                std::fill(f, f + k + 1, 0.0);
                vn1[j] = vn2[j] = std::sqrt(dot(c + rk + 1, c + rk + 1, m - rk - 1));
            }
        }
        const int r0 = off + k;
        /* the block's reflectors reach the columns below the stop norm */
        for (int j = r0; j < n; j++)
            if (done[j] >= 0 && done[j] < r0) {
                apply_reflectors(A + (size_t)j * ld, A, ld, m, tau.data(), off, done[j], r0);
                done[j] = r0;
            }
        /* stopped inside the block: rows 0..r0-1 (R11, R12) are final already */
        if (k < nb) return r0;
        /* the trailing matrix: A(r0:m, j) -= V(r0:m, 0:k) F(j, 0:k)^T, live columns j */
        live.clear();
        for (int j = r0; j < n; j++)
            if (done[j] < 0) live.push_back(j);
        const int nl = (int)live.size();
        int q = 0;
        for (; q + 2 <= nl; q += 2)
            apply_block(A + (size_t)live[q] * ld, &F[(size_t)live[q] * kQrBlock], A + (size_t)live[q + 1] * ld,
                        &F[(size_t)live[q + 1] * kQrBlock], V, ld, k, r0, m);
        if (q < nl) apply_block(A + (size_t)live[q] * ld, &F[(size_t)live[q] * kQrBlock], nullptr, nullptr, V, ld, k, r0, m);
        off = r0;
    }
    return kmax;
}

/* ID over the rows of a row-major nrow x ncol matrix A: A ~= U * A(J, :)
 * (H2P-ERI src/H2E_ID_compress.c:433-576). A row-major is A^T column-major,
 * so pivoted QR on that view picks skeleton rows. */
void id_compress(H2E_dense_mat_p A, double rel_tol, H2E_dense_mat_p *U_out, H2E_int_vec_p J)
{
    const int nrow = A->nrow, ncol = A->ncol, ld = A->ld;
    std::vector<int> p(std::max(nrow, 1));
    int r = (nrow > 0 && ncol > 0) ? pivoted_qr(A->data, ncol, nrow, ld, rel_tol, p.data()) : 0;
    if (r == 0) {
        J->length = 0;
        if (U_out) {
            H2E_dense_mat_p U = dmat_new(0, 0);
            U->nrow = nrow;
            U->ncol = 0;
            U->ld = 0;
            *U_out = U;
        }
        return;
    }
    /* sorted skeleton rows and, for each, its pivot position */
    std::vector<std::pair<int, int>> sk(r);
    for (int k = 0; k < r; k++) sk[k] = {p[k], k};
    std::sort(sk.begin(), sk.end());
    ivec_reserve(J, r);
    for (int k = 0; k < r; k++) J->data[k] = sk[k].first;
    J->length = r;
    if (U_out == nullptr) return;
    /* E = R11^{-1} R12, R11 r x r upper triangular, R12 r x (nrow - r); column-major with ld */
    const int ne = nrow - r;
    double *R = A->data;
    /* back substitution by columns of R11 (contiguous), two columns of E at once */
    int ce = 0;
    for (; ce + 2 <= ne; ce += 2) {
        double *x = R + (size_t)(r + ce) * ld, *y = x + ld;
        for (int i = r - 1; i >= 0; i--) {
            const double *ri = R + (size_t)i * ld;
            const double xi = x[i] / ri[i], yi = y[i] / ri[i];
            x[i] = xi;
            y[i] = yi;
            for (int k = 0; k < i; k++) {
                x[k] -= ri[k] * xi;
                y[k] -= ri[k] * yi;
            }
        }
    }
    for (; ce < ne; ce++) {
        double *x = R + (size_t)(r + ce) * ld;
        for (int i = r - 1; i >= 0; i--) {
            const double *ri = R + (size_t)i * ld;
            const double xi = x[i] / ri[i];
            x[i] = xi;
            for (int k = 0; k < i; k++) x[k] -= ri[k] * xi;
        }
    }
    H2E_dense_mat_p U = dmat_new(nrow, r);
    std::vector<int> sorted_pos(r);      /* pivot position -> sorted column */
    for (int k = 0; k < r; k++) sorted_pos[sk[k].second] = k;
    for (int k = 0; k < nrow; k++) {
        int row = p[k];
        double *u = U->data + (size_t)row * r;
        if (k < r) {
            std::memset(u, 0, sizeof(double) * r);
            u[sorted_pos[k]] = 1.0;
        } else {
            const double *e = R + (size_t)k * ld;   /* column r + (k - r) of E */
            for (int c = 0; c < r; c++) u[c] = e[sk[c].second];
        }
    }
    *U_out = U;
}

/* ---------------------------------------------------------------------- */
/* Helpers for the U construction                                          */
/* ---------------------------------------------------------------------- */

namespace {

struct Rng {   /* splitmix64 */
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
};

/* Sparse random k x n matrix with min(max_nnz_col, k) entries +-1 per column,
 * stored as n rows (columns of the matrix) of column indices
 * (H2P-ERI src/H2ERI_utils.c:49-96). */
struct Sketch {
    int nnz_col = 0, n = 0;
    std::vector<double> val;
    std::vector<int> col;
};

void gen_sketch(int max_nnz_col, int k, int n, Rng &rng, Sketch &s)
{
    s.nnz_col = std::min(max_nnz_col, k);
    s.n = n;
    s.val.resize((size_t)n * s.nnz_col);
    s.col.resize((size_t)n * s.nnz_col);
    for (auto &v : s.val) v = (rng.next() & 1) ? 1.0 : -1.0;
    std::vector<char> flag(std::max(k, 1), 0);
    for (int i = 0; i < n; i++) {
        int *c = s.col.data() + (size_t)i * s.nnz_col;
        int cnt = 0;
        while (cnt < s.nnz_col) {
            int x = (int)(rng.next() % (uint64_t)k);
            if (!flag[x]) { flag[x] = 1; c[cnt++] = x; }
        }
        for (int j = 0; j < s.nnz_col; j++) flag[c[j]] = 0;
    }
}

/* y (m x n, ldy) = x (m x k, ldx) * S (src/H2ERI_utils.c:99-118) */
void sketch_apply(int m, const Sketch &s, const double *x, int ldx, double *y, int ldy)
{
    for (int i = 0; i < m; i++) {
        const double *xi = x + (size_t)i * ldx;
        double *yi = y + (size_t)i * ldy;
        for (int j = 0; j < s.n; j++) {
            double r = 0.0;
            const int *c = s.col.data() + (size_t)j * s.nnz_col;
            const double *v = s.val.data() + (size_t)j * s.nnz_col;
            for (int l = 0; l < s.nnz_col; l++) r += v[l] * xi[c[l]];
            yi[j] = r;
        }
    }
}

/* Proxy points: nlayer scaled copies of a uniform grid on the surface of
 * [-1,1]^3 between radii r1 and r2 (src/H2ERI_build_H2.c:25-103).
 * Output pp = [x(0..n) | y(0..n) | z(0..n)]. */
void proxy_points(double r1, double r2, int nlayer, int npts_layer, std::vector<double> &pp, int &npts)
{
    int nface = npts_layer / 6;
    int naxis = (int)std::ceil(std::sqrt((double)nface));
    int nl = 6 * naxis * naxis;
    npts = nlayer * nl;
    pp.assign((size_t)npts * 3, 0.0);
    double *x = pp.data(), *y = x + npts, *z = y + npts;
    double hstep = 2.0 / (double)(naxis + 1);
    int idx = 0;
    for (int i = 0; i < naxis; i++) {
        double hi = hstep * (i + 1) - 1.0;
        for (int j = 0; j < naxis; j++) {
            double hj = hstep * (j + 1) - 1.0;
            const double f[6][3] = {{hi, hj, -1.0}, {hi, hj, 1.0}, {hi, -1.0, hj},
                                    {hi, 1.0, hj}, {-1.0, hi, hj}, {1.0, hi, hj}};
            for (int q = 0; q < 6; q++) { x[idx] = f[q][0]; y[idx] = f[q][1]; z[idx] = f[q][2]; idx++; }
        }
    }
    for (int l = 1; l < nlayer; l++) {
        std::memcpy(x + l * nl, x, sizeof(double) * nl);
        std::memcpy(y + l * nl, y, sizeof(double) * nl);
        std::memcpy(z + l * nl, z, sizeof(double) * nl);
    }
    int nl1 = std::max(nlayer - 1, 1);
    double dr = ((r2 - r1) / r1) / (double)nl1;
    for (int l = 0; l < nlayer; l++) {
        double r = r1 * (1.0 + l * dr);
        for (int j = 0; j < nl; j++) { x[l * nl + j] *= r; y[l * nl + j] *= r; z[l * nl + j] *= r; }
    }
}

/* Far-field SSPs whose extents overlap each node's near field
 * (src/H2ERI_build_H2.c:115-259). */
void calc_ovlp_ff_idx(H2ERI_p h)
{
    const int n_node = h->n_node, n_point = h->n_point;
    const double *cx = h->sp_center, *cy = cx + n_point, *cz = cy + n_point, *ext = h->sp_extent;
    h->ovlp_ff_idx = (H2E_int_vec_p *)std::malloc(sizeof(H2E_int_vec_p) * n_node);
    for (int i = 0; i < n_node; i++) h->ovlp_ff_idx[i] = ivec_new(n_point);
    H2E_int_vec_p root = h->ovlp_ff_idx[h->root_idx];
    for (int i = 0; i < n_point; i++) root->data[i] = i;
    root->length = n_point;
    for (int lv = 0; lv < h->max_level; lv++) {
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = h->level_nodes[lv * h->n_leaf_node + j];
            H2E_int_vec_p par = h->ovlp_ff_idx[node];
            for (int k = 0; k < h->n_child[node]; k++) {
                int c = h->children[node * h->max_child + k];
                const double *eb = h->enbox + 6 * c;
                double ec[3] = {eb[0] + 0.5 * eb[3], eb[1] + 0.5 * eb[4], eb[2] + 0.5 * eb[5]};
                double sup = 0.5 + H2G_ALPHA_SUP;
                double sl[3] = {sup * eb[3], sup * eb[4], sup * eb[5]};
                H2E_int_vec_p out = h->ovlp_ff_idx[c];
                for (int l = 0; l < par->length; l++) {
                    int f = par->data[l];
                    double e = ext[f];
                    double rel[3] = {cx[f] - ec[0] + sl[0] - e, cy[f] - ec[1] + sl[1] - e, cz[f] - ec[2] + sl[2] - e};
                    bool adm_any = false;
                    for (int d = 0; d < 3; d++) {
                        bool left = rel[d] < 0, right = rel[d] >= 0;
                        bool adm_l = std::fabs(rel[d]) >= 2.0 * e - 1e-8;
                        bool adm_r = std::fabs(rel[d]) >= 2.0 * sl[d] - 1e-8;
                        if ((left && adm_l) || (right && adm_r)) adm_any = true;
                    }
                    if (!adm_any) out->data[out->length++] = f;
                }
            }
        }
    }
    std::vector<int> tmp(n_point);
    for (int lv = h->min_adm_level; lv <= h->max_level; lv++) {
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = h->level_nodes[lv * h->n_leaf_node + j];
            const double *eb = h->enbox + 6 * node;
            double ec[3] = {eb[0] + 0.5 * eb[3], eb[1] + 0.5 * eb[4], eb[2] + 0.5 * eb[5]};
            double ac = 0.5 + H2G_ALPHA_H2;
            double al[3] = {ac * eb[3], ac * eb[4], ac * eb[5]};
            H2E_int_vec_p v = h->ovlp_ff_idx[node];
            int cnt = 0;
            for (int l = 0; l < v->length; l++) {
                int f = v->data[l];
                if (std::fabs(cx[f] - ec[0]) > al[0] || std::fabs(cy[f] - ec[1]) > al[1] ||
                    std::fabs(cz[f] - ec[2]) > al[2])
                    tmp[cnt++] = f;
            }
            std::memcpy(v->data, tmp.data(), sizeof(int) * cnt);
            v->length = cnt;
        }
    }
}

/* Given bf-pair row indices (ascending, relative to the concatenation of the
 * SSPs in sp_idx), find the SSPs that contain them and the row indices inside
 * the concatenation of just those SSPs (src/H2ERI_build_H2.c:271-335).
 * pair_pos receives positions into sp_idx. */
void extract_sp_idx(H2ERI_p h, const int *row_idx, int n_row, const int *sp_idx, int n_sp,
                    std::vector<int> &pair_pos, std::vector<int> &row_new)
{
    std::vector<int> off(n_sp + 1, 0), which(n_row), flag(n_sp, 0);
    for (int i = 0; i < n_sp; i++) off[i + 1] = off[i] + h->sp_nbfp[sp_idx[i]];
    int j = 0;
    for (int i = 0; i < n_row; i++) {
        int x = row_idx[i];
        /* rows are ascending, but restart the scan to be safe for unsorted input */
        if (j >= n_sp || x < off[j]) j = 0;
        while (j < n_sp && !(off[j] <= x && x < off[j + 1])) j++;
        which[i] = j;
        flag[j] = 1;
    }
    pair_pos.clear();
    std::vector<int> newpos(n_sp, -1);
    for (int i = 0; i < n_sp; i++)
        if (flag[i]) { newpos[i] = (int)pair_pos.size(); pair_pos.push_back(i); }
    std::vector<int> noff(pair_pos.size() + 1, 0);
    for (size_t i = 0; i < pair_pos.size(); i++) noff[i + 1] = noff[i] + h->sp_nbfp[sp_idx[pair_pos[i]]];
    row_new.resize(n_row);
    for (int i = 0; i < n_row; i++) row_new[i] = row_idx[i] - off[which[i]] + noff[newpos[which[i]]];
}

int sum_nbfp(H2ERI_p h, const int *idx, int n)
{
    int s = 0;
    for (int i = 0; i < n; i++) s += h->sp_nbfp[idx[i]];
    return s;
}

bool setup_verbose();

/* Dense block -> dense or low-rank storage (src/H2ERI_build_H2.c:843-903). */
H2E_dense_mat_p compress_block(H2E_dense_mat_p blk, double rel_tol)
{
    const int nr = blk->nrow, nc = blk->ncol;
    H2E_dense_mat_p work = dmat_new(nr, nc);
    if ((size_t)nr * nc > 0) std::memcpy(work->data, blk->data, sizeof(double) * (size_t)nr * nc);
    H2E_int_vec_p J = ivec_new(std::max(nr, 1));
    H2E_dense_mat_p U = nullptr;
    id_compress(work, rel_tol, &U, J);
    dmat_free(&work);
    int r = J->length;
    int old_size = nr * nc, new_size = (nr + nc) * r;
    H2E_dense_mat_p res;
    if (new_size > old_size * 4 / 5) {
        res = dmat_new(nr, nc);
        if (old_size > 0) std::memcpy(res->data, blk->data, sizeof(double) * (size_t)old_size);
    } else {
        res = dmat_new(1, new_size);
        res->nrow = nr;
        res->ncol = nc;
        res->ld = -r;
        double *Up = res->data, *Vt = Up + (size_t)nr * r;
        std::memcpy(Up, U->data, sizeof(double) * (size_t)nr * r);
        for (int l = 0; l < nc; l++)
            for (int k = 0; k < r; k++) Vt[(size_t)l * r + k] = blk->data[(size_t)J->data[k] * nc + l];
    }
    dmat_free(&U);
    ivec_free(&J);
    return res;
}

/* Integer COO -> CSR with columns sorted per row (src/H2ERI_utils.c:121-146). */
void coo_to_csr(int nrow, int nnz, const int *row, const int *col, const int *val, int *rp, int *ci, int *cv)
{
    std::memset(rp, 0, sizeof(int) * (nrow + 1));
    for (int i = 0; i < nnz; i++) rp[row[i] + 1]++;
    for (int i = 1; i <= nrow; i++) rp[i] += rp[i - 1];
    std::vector<int> pos(rp, rp + nrow);
    for (int i = 0; i < nnz; i++) {
        int k = pos[row[i]]++;
        ci[k] = col[i];
        cv[k] = val[i];
    }
    for (int r = 0; r < nrow; r++) {
        std::vector<std::pair<int, int>> e;
        for (int k = rp[r]; k < rp[r + 1]; k++) e.push_back({ci[k], cv[k]});
        std::sort(e.begin(), e.end());
        for (int k = rp[r]; k < rp[r + 1]; k++) { ci[k] = e[k - rp[r]].first; cv[k] = e[k - rp[r]].second; }
    }
}

/* ERI sub-block: rows = selected bf pairs of the bra SSPs, cols = selected
 * bf pairs of the ket SSPs. sel_row/sel_col index into the concatenations of
 * all bf pairs of bra / ket (nullptr = all). Row-major nrow x ncol. */
void eri_block(H2ERI_p h, const int *bra, int nbra, const int *ket, int nket,
               const int *sel_row, int nrow, const int *sel_col, int ncol, double *out)
{
    const int full_r = sum_nbfp(h, bra, nbra), full_c = sum_nbfp(h, ket, nket);
    std::vector<double> full((size_t)full_r * full_c);
    eri_pairs_to_mat(h, nbra, bra, nket, ket, full.data(), full_c);
    for (int r = 0; r < nrow; r++) {
        const double *src = full.data() + (size_t)(sel_row ? sel_row[r] : r) * full_c;
        double *dst = out + (size_t)r * ncol;
        if (sel_col)
            for (int c = 0; c < ncol; c++) dst[c] = src[sel_col[c]];
        else
            std::memcpy(dst, src, sizeof(double) * ncol);
    }
}

/* Shell pairs of near-field block i: a leaf's diagonal block (bra = ket =
 * its shell pairs, symmetric) or an inadmissible pair's block. */
void d_block_lists(H2ERI_p h, int i, std::vector<int> &bra, std::vector<int> &ket, bool &sym)
{
    const int n_leaf = h->n_leaf_node;
    bra.clear();
    ket.clear();
    int n0, n1;
    if (i < n_leaf) {
        n0 = n1 = h->height_nodes[i];
        sym = true;
    } else {
        n0 = h->r_inadm_pairs[2 * (i - n_leaf)];
        n1 = h->r_inadm_pairs[2 * (i - n_leaf) + 1];
        sym = false;
    }
    for (int k = h->pt_cluster[2 * n0]; k <= h->pt_cluster[2 * n0 + 1]; k++) bra.push_back(k);
    for (int k = h->pt_cluster[2 * n1]; k <= h->pt_cluster[2 * n1 + 1]; k++) ket.push_back(k);
}

/* Dense near-field block i with the host engine. Diagonal blocks are
 * symmetric; only their upper shell-pair triangle is evaluated and mirrored. */
void d_block_host(H2ERI_p h, int i, H2E_dense_mat_p blk)
{
    if (i < h->n_leaf_node) {
        int node = h->height_nodes[i];
        int ps = h->pt_cluster[2 * node], pe = h->pt_cluster[2 * node + 1];
        int n = blk->nrow;
        std::vector<double> buf(15 * 15 * 15 * 15);
        for (int a = ps; a <= pe; a++) {
            int ra = h->sp_bfp_sidx[a] - h->sp_bfp_sidx[ps], na = h->sp_nbfp[a];
            const h2g_pair *pa = sp_pair(h, a);
            for (int b = a; b <= pe; b++) {
                int rb = h->sp_bfp_sidx[b] - h->sp_bfp_sidx[ps], nb = h->sp_nbfp[b];
                h2g_eri_quartet(pa, sp_pair(h, b), buf.data());
                for (int x = 0; x < na; x++)
                    for (int y = 0; y < nb; y++) {
                        double v = buf[(size_t)x * nb + y];
                        blk->data[(size_t)(ra + x) * n + rb + y] = v;
                        blk->data[(size_t)(rb + y) * n + ra + x] = v;
                    }
            }
        }
    } else {
        std::vector<int> bra, ket;
        bool sym;
        d_block_lists(h, i, bra, ket, sym);
        eri_pairs_to_mat(h, (int)bra.size(), bra.data(), (int)ket.size(), ket.data(), blk->data, blk->ncol);
    }
}

/* H2G_SETUP_VERBOSE=1: timings of the set-up's phases on stderr. */
bool setup_verbose()
{
    const char *v = std::getenv("H2G_SETUP_VERBOSE");
    return v != nullptr && v[0] == '1';
}

/* The set-up's ERI blocks on the GPU (when gpu_eri_usable(): a CUDA device
 * and H2G_SETUP_GPU not 0): the structure's shell pairs, uploaded on first
 * use and kept until the set-up ends; nullptr means the host engine. */
struct SetupEri {
    H2ERI_p h = nullptr;
    EriSet *es = nullptr;
    bool failed = false;
};
static thread_local SetupEri g_seri;   /* per calling thread: set-ups of different structures may run at once */

EriSet *setup_eri(H2ERI_p h)
{
    if (g_seri.h == h) return g_seri.failed ? nullptr : g_seri.es;
    if (g_seri.es) gpu_eri_free(g_seri.es);
    g_seri = SetupEri();
    g_seri.h = h;
    if (!gpu_eri_usable()) { g_seri.failed = true; return nullptr; }
    std::vector<const h2g_pair *> pairs(h->num_sp);
    for (int i = 0; i < h->num_sp; i++) pairs[i] = sp_pair(h, i);
    if (gpu_eri_create(h->num_sp, pairs.data(), &g_seri.es) != 0) {
        g_seri.failed = true;
        g_seri.es = nullptr;
    }
    return g_seri.es;
}

void setup_eri_failed(H2ERI_p h)
{
    std::fprintf(stderr, "h2eri_gb300: GPU integral blocks failed (%s); the host engine takes over\n",
                 H2ERI_gpu_last_error());
    if (g_seri.h == h) g_seri.failed = true;
}

void setup_eri_end()
{
    if (g_seri.es) gpu_eri_free(g_seri.es);
    g_seri = SetupEri();
}

/* Groups of ERI blocks evaluated on the GPU one group ahead of their use on
 * the host: while use(g, reqs) runs for group g in the calling thread
 * (compression), a worker thread evaluates group g + 1. prep(g, reqs) fills
 * the requests of group g. Returns the number of groups used; a GPU failure
 * stops the pipeline, and discard(g, reqs) releases a prepared group that
 * was not used. */
template <class Req, class Eval, class Prep, class Use, class Discard>
int gpu_pipeline(H2ERI_p h, int n_groups, Eval eval, Prep prep, Use use, Discard discard)
{
    if (n_groups == 0) return 0;
    std::vector<Req> cur, nxt;
    prep(0, cur);
    const double t0 = wtime();
    int rc = eval(cur);
    double t_gpu_first = wtime() - t0, t_use = 0.0, t_wait = 0.0;
    int g = 0;
    for (; g < n_groups; g++) {
        if (rc != 0) {
            discard(g, cur);
            setup_eri_failed(h);
            break;
        }
        int rc_next = 0;
        std::string msg_next;   /* error messages are per thread */
        std::thread th;
        if (g + 1 < n_groups) {
            nxt.clear();
            prep(g + 1, nxt);
            th = std::thread([&] {
                rc_next = eval(nxt);
                if (rc_next) msg_next = H2ERI_gpu_last_error();
            });
        }
        const double tu = wtime();
        use(g, cur);
        const double tw = wtime();
        if (th.joinable()) th.join();
        t_use += tw - tu;
        t_wait += wtime() - tw;
        std::swap(cur, nxt);
        rc = rc_next;
        if (rc) std::fprintf(stderr, "h2eri_gb300: GPU integral blocks: %s\n", msg_next.c_str());
    }
    if (setup_verbose())
        std::fprintf(stderr, "gpu pipeline: %d groups, first group on the GPU %.3f s, host use %.3f s, waiting for "
                     "the GPU %.3f s\n", g, t_gpu_first, t_use, t_wait);
    return g;
}

/* ---- nested bases U and skeleton sets (src/H2ERI_build_H2.c:351-827) ----
 *
 * Per node, from the leaves up: the candidate rows (all bf pairs of a leaf,
 * the children's skeleton rows otherwise), a matrix of their integrals with
 * proxy point charges around the node box and with the overlapping
 * far-field shell pairs, each side reduced to nrow columns by a sparse sign
 * sketch, then an interpolative decomposition of the column-normalised
 * candidate rows. The integrals and sketches run on the GPU when the set-up
 * may use it (gpu_eri_usable), a level's nodes in groups, the next group on
 * the GPU while the host decomposes the current one; otherwise on the host
 * engine. */

/* One node's inputs and its sketched matrix (nrow_blk x 2 nrow_blk). */
struct UNode {
    int node = -1;
    std::vector<int> pair_idx, row_idx;
    int nrow_blk = 0;
    std::vector<double> pp;   /* the proxy points a sketch uses: [x | y | z], cnt each */
    int cnt = 0;
    Sketch s1, s2;            /* columns into the points / into ff1's bf pairs */
    std::vector<int> ff1;     /* far-field shell pairs a sketch uses */
    int ff_ncol1 = 0;
    std::vector<double> A;
};

/* Candidate rows, proxy points, far-field pairs and both sketches of node
 * (the host path's order of random draws: potentials' sketch first). */
void u_prep(H2ERI_p h, int node, const std::vector<int> &skel, UNode &w)
{
    w.node = node;
    const int nch = h->n_child[node];
    w.pair_idx.clear();
    w.row_idx.clear();
    /* (1) candidate rows of this node */
    if (nch == 0) {
        for (int k = h->pt_cluster[2 * node]; k <= h->pt_cluster[2 * node + 1]; k++)
            w.pair_idx.push_back(h->index_seq[k]);
        int nb = sum_nbfp(h, w.pair_idx.data(), (int)w.pair_idx.size());
        for (int k = 0; k < nb; k++) w.row_idx.push_back(k);
    } else {
        int roff = 0;
        for (int k = 0; k < nch; k++) {
            int c = h->children[node * h->max_child + k];
            for (int t = 0; t < h->J_pair[c]->length; t++) w.pair_idx.push_back(h->J_pair[c]->data[t]);
            for (int t = 0; t < h->J_row[c]->length; t++) w.row_idx.push_back(h->J_row[c]->data[t] + roff);
            roff += sum_nbfp(h, h->J_pair[c]->data, h->J_pair[c]->length);
        }
    }
    /* (2) proxy points around the node box */
    const double *eb = h->enbox + 6 * node;
    double width = eb[3], extent = h->box_extent[node];
    double r1 = width * (0.5 + H2G_ALPHA_SUP), r2 = width * (0.5 + extent);
    int nlayer = std::max(1, 1 + (int)std::ceil((extent - H2G_ALPHA_SUP) * (h->pp_nlayer_ext - 1)));
    int num_pp;
    proxy_points(r1, r2, nlayer, h->pp_npts_layer, w.pp, num_pp);
    double *ppx = w.pp.data(), *ppy = ppx + num_pp, *ppz = ppy + num_pp;
    for (int k = 0; k < num_pp; k++) {
        ppx[k] += eb[0] + 0.5 * eb[3];
        ppy[k] += eb[1] + 0.5 * eb[4];
        ppz[k] += eb[2] + 0.5 * eb[5];
    }
    /* (3) far-field SSPs that are still skeletons */
    std::vector<int> ff;
    H2E_int_vec_p ov = h->ovlp_ff_idx[node];
    for (int k = 0; k < ov->length; k++)
        if (skel[ov->data[k]]) ff.push_back(ov->data[k]);
    w.nrow_blk = sum_nbfp(h, w.pair_idx.data(), (int)w.pair_idx.size());
    const int ff_ncol = sum_nbfp(h, ff.data(), (int)ff.size());
    Rng rng(0x5eed0000ULL + (uint64_t)node * 7919ULL);
    /* (4) sketch of the proxy-point potentials; only the points it uses stay */
    gen_sketch(16, num_pp, w.nrow_blk, rng, w.s1);
    {
        std::vector<int> map(num_pp, -1);
        for (int c : w.s1.col) map[c] = 1;
        int cnt = 0;
        for (int k = 0; k < num_pp; k++)
            if (map[k] >= 0) {
                map[k] = cnt;
                ppx[cnt] = ppx[k]; ppy[cnt] = ppy[k]; ppz[cnt] = ppz[k];
                cnt++;
            }
        for (auto &c : w.s1.col) c = map[c];
        std::vector<double> q((size_t)3 * cnt);
        std::memcpy(q.data(), ppx, sizeof(double) * cnt);
        std::memcpy(q.data() + cnt, ppy, sizeof(double) * cnt);
        std::memcpy(q.data() + 2 * cnt, ppz, sizeof(double) * cnt);
        w.pp.swap(q);
        w.cnt = cnt;
    }
    /* (5) sketch of the ERIs with the far-field SSPs; only the SSPs it uses stay */
    gen_sketch(16, ff_ncol, w.nrow_blk, rng, w.s2);
    {
        std::vector<int> used(std::max(ff_ncol, 1), -1);
        for (int c : w.s2.col) used[c] = 1;
        std::vector<int> cup;
        for (int k = 0; k < ff_ncol; k++)
            if (used[k] >= 0) { used[k] = (int)cup.size(); cup.push_back(k); }
        std::vector<int> pos, cup_new;
        extract_sp_idx(h, cup.data(), (int)cup.size(), ff.data(), (int)ff.size(), pos, cup_new);
        w.ff1.resize(pos.size());
        for (size_t k = 0; k < pos.size(); k++) w.ff1[k] = ff[pos[k]];
        for (auto &c : w.s2.col) c = cup_new[used[c]];
        w.ff_ncol1 = sum_nbfp(h, w.ff1.data(), (int)w.ff1.size());
    }
    w.A.assign((size_t)w.nrow_blk * 2 * w.nrow_blk, 0.0);
}

/* The node's sketched matrix on the host engine. */
void u_integrals_host(H2ERI_p h, UNode &w, double &t_nai, double &t_eri)
{
    const int nrow_blk = w.nrow_blk, ncol_blk = 2 * nrow_blk, cnt = w.cnt;
    const double tp0 = wtime();
    {
        std::vector<double> Apot((size_t)nrow_blk * std::max(cnt, 1));
        nai_pairs_to_mat(h, (int)w.pair_idx.size(), w.pair_idx.data(), cnt, w.pp.data(), w.pp.data() + cnt,
                         w.pp.data() + 2 * cnt, Apot.data(), cnt);
        sketch_apply(nrow_blk, w.s1, Apot.data(), cnt, w.A.data(), ncol_blk);
    }
    const double tp1 = wtime();
    {
        std::vector<double> Aff((size_t)15 * 15 * std::max(w.ff_ncol1, 1));
        int rcnt = 0;
        for (size_t k = 0; k < w.pair_idx.size(); k++) {
            int nb = h->sp_nbfp[w.pair_idx[k]];
            eri_pairs_to_mat(h, 1, &w.pair_idx[k], (int)w.ff1.size(), w.ff1.data(), Aff.data(), w.ff_ncol1);
            sketch_apply(nb, w.s2, Aff.data(), w.ff_ncol1, w.A.data() + (size_t)rcnt * ncol_blk + nrow_blk, ncol_blk);
            rcnt += nb;
        }
    }
    const double tp2 = wtime();
    #pragma omp atomic
    t_nai += tp1 - tp0;
    #pragma omp atomic
    t_eri += tp2 - tp1;
}

/* (6) normalise columns, keep candidate rows, ID; (7) skeleton SSPs and rows. */
void u_finish(H2ERI_p h, UNode &w)
{
    const int nrow_blk = w.nrow_blk, ncol_blk = 2 * nrow_blk, node = w.node;
    std::vector<double> &Ablk = w.A;
    std::vector<double> inv(ncol_blk, 0.0);
    for (int c = 0; c < ncol_blk; c++) {
        double s = 0.0;
        for (int r = 0; r < nrow_blk; r++) s += Ablk[(size_t)r * ncol_blk + c] * Ablk[(size_t)r * ncol_blk + c];
        inv[c] = (s > 0.0) ? 1.0 / std::sqrt(s) : 0.0;
    }
    const int nsel = (int)w.row_idx.size();
    H2E_dense_mat_p A = dmat_new(nsel, ncol_blk);
    for (int r = 0; r < nsel; r++) {
        const double *src = Ablk.data() + (size_t)w.row_idx[r] * ncol_blk;
        double *dst = A->data + (size_t)r * ncol_blk;
        for (int c = 0; c < ncol_blk; c++) dst[c] = src[c] * inv[c];
    }
    H2E_int_vec_p J = ivec_new(std::max(nsel, 1));
    H2E_dense_mat_p U = nullptr;
    id_compress(A, h->QR_stop_tol, &U, J);
    dmat_free(&A);
    h->U[node] = U;
    std::vector<int> sub_row(J->length);
    for (int k = 0; k < J->length; k++) sub_row[k] = w.row_idx[J->data[k]];
    std::vector<int> pos, rnew;
    extract_sp_idx(h, sub_row.data(), (int)sub_row.size(), w.pair_idx.data(), (int)w.pair_idx.size(), pos, rnew);
    H2E_int_vec_p jp = ivec_new(std::max((int)pos.size(), 1));
    H2E_int_vec_p jr = ivec_new(std::max((int)rnew.size(), 1));
    for (size_t k = 0; k < pos.size(); k++) jp->data[k] = w.pair_idx[pos[k]];
    jp->length = (int)pos.size();
    for (size_t k = 0; k < rnew.size(); k++) jr->data[k] = rnew[k];
    jr->length = (int)rnew.size();
    h->J_pair[node] = jp;
    h->J_row[node] = jr;
    ivec_free(&J);
    std::vector<double>().swap(w.A);
}

/* The GPU request of a prepared node (host pointers into w). */
UReq u_request(UNode &w)
{
    UReq q;
    q.bra = w.pair_idx.data();
    q.nbra = (int)w.pair_idx.size();
    q.ket = w.ff1.data();
    q.nket = (int)w.ff1.size();
    q.px = w.pp.data();
    q.py = w.pp.data() + w.cnt;
    q.pz = w.pp.data() + 2 * w.cnt;
    q.npt = w.cnt;
    q.s1_col = w.s1.col.data();
    q.s1_val = w.s1.val.data();
    q.s1_nnz = w.s1.nnz_col;
    q.s2_col = w.s2.col.data();
    q.s2_val = w.s2.val.data();
    q.s2_nnz = w.s2.nnz_col;
    q.out = w.A.data();
    q.ld = 2 * w.nrow_blk;
    return q;
}

void build_UJ_proxy(H2ERI_p h)
{
    const int n_node = h->n_node, n_point = h->n_point, n_leaf = h->n_leaf_node;
    const int max_level = h->max_level, min_adm = h->min_adm_level;
    h->n_UJ = n_node;
    h->U = (H2E_dense_mat_p *)std::calloc(n_node, sizeof(H2E_dense_mat_p));
    h->J_pair = (H2E_int_vec_p *)std::calloc(n_node, sizeof(H2E_int_vec_p));
    h->J_row = (H2E_int_vec_p *)std::calloc(n_node, sizeof(H2E_int_vec_p));
    std::vector<int> skel(n_point, 1);
    std::vector<std::vector<int>> lvl_leaf(max_level + 1);
    for (int i = 0; i < n_leaf; i++) {
        int leaf = h->height_nodes[i];
        for (int lv = h->node_level[leaf] + 1; lv <= max_level; lv++) lvl_leaf[lv].push_back(leaf);
    }
    calc_ovlp_ff_idx(h);
    /* thread seconds per phase (reported with H2G_SETUP_VERBOSE=1) */
    double t_prep = 0.0, t_nai = 0.0, t_eri = 0.0, t_id = 0.0, t_gpu_wall = 0.0;
    int n_gpu = 0;

    for (int lv = max_level; lv >= min_adm; lv--) {
        const int nlv = h->level_n_node[lv];
        const int *lnodes = h->level_nodes + lv * n_leaf;
        std::vector<UNode> W(nlv);
        const double tp = wtime();
        #pragma omp parallel for schedule(dynamic, 1)
        for (int jn = 0; jn < nlv; jn++) u_prep(h, lnodes[jn], skel, W[jn]);
        t_prep += wtime() - tp;
        int done = 0;
        if (EriSet *es = setup_eri(h)) {
            /* groups of at most 2^27 doubles of unsketched integrals (2^25
             * for the first, so that the host starts early) */
            std::vector<int> gstart(1, 0);
            long long tot = 0;
            for (int jn = 0; jn < nlv; jn++) {
                const long long n = (long long)W[jn].nrow_blk * (W[jn].cnt + W[jn].ff_ncol1);
                if (jn > gstart.back() && tot + n > (gstart.size() == 1 ? (1LL << 25) : (1LL << 27))) {
                    gstart.push_back(jn);
                    tot = 0;
                }
                tot += n;
            }
            gstart.push_back(nlv);
            const int n_groups = (int)gstart.size() - 1;
            auto prep = [&](int g, std::vector<UReq> &reqs) {
                for (int jn = gstart[g]; jn < gstart[g + 1]; jn++)
                    if (W[jn].nrow_blk > 0) reqs.push_back(u_request(W[jn]));
            };
            auto use = [&](int g, std::vector<UReq> &) {
                const double t0 = wtime();
                #pragma omp parallel for schedule(dynamic, 1)
                for (int jn = gstart[g]; jn < gstart[g + 1]; jn++) u_finish(h, W[jn]);
                t_id += wtime() - t0;
            };
            auto discard = [&](int, std::vector<UReq> &) {};
            const double tg = wtime();
            const int used = gpu_pipeline<UReq>(
                h, n_groups, [es](std::vector<UReq> &r) { return gpu_u_blocks(es, r); }, prep, use, discard);
            t_gpu_wall += wtime() - tg;
            done = gstart[used];
            n_gpu += done;
        }
        #pragma omp parallel for schedule(dynamic, 1)
        for (int jn = done; jn < nlv; jn++) {
            u_integrals_host(h, W[jn], t_nai, t_eri);
            const double t0 = wtime();
            u_finish(h, W[jn]);
            #pragma omp atomic
            t_id += wtime() - t0;
        }
        /* skeleton flags for the next level up */
        std::fill(skel.begin(), skel.end(), 0);
        for (int jn = 0; jn < nlv; jn++) {
            int node = lnodes[jn];
            for (int k = 0; k < h->J_pair[node]->length; k++) skel[h->J_pair[node]->data[k]] = 1;
        }
        for (int leaf : lvl_leaf[lv])
            for (int k = h->pt_cluster[2 * leaf]; k <= h->pt_cluster[2 * leaf + 1]; k++) skel[k] = 1;
    }
    if (setup_verbose())
        std::fprintf(stderr, "build_U: %d nodes with GPU integrals (wall %.2f s incl. the decompositions between), "
                     "host: preparation %.2f s wall, proxy-point potentials %.2f, far-field ERI %.2f thread s, ID "
                     "%.2f s (wall on the GPU path, thread s on the host path)\n", n_gpu, t_gpu_wall, t_prep, t_nai,
                     t_eri, t_id);
    for (int i = 0; i < n_node; i++) {
        if (h->U[i] == nullptr) {
            h->U[i] = dmat_new(1, 1);
            h->U[i]->nrow = 0;
            h->U[i]->ncol = 0;
            h->U[i]->ld = 0;
        } else {
            size_t nr = h->U[i]->nrow, nc = h->U[i]->ncol;
            h->mat_size[U_SIZE_IDX] += nr * nc;
            h->mat_size[MV_FWD_SIZE_IDX] += nr * nc + nr + nc;
            h->mat_size[MV_BWD_SIZE_IDX] += nr * nc + nr + nc;
        }
        if (h->J_row[i] == nullptr) h->J_row[i] = ivec_new(1);
        if (h->J_pair[i] == nullptr) h->J_pair[i] = ivec_new(1);
    }
}

/* Coupling blocks (src/H2ERI_build_H2.c:910-1152). */
void build_B(H2ERI_p h)
{
    const int n_pair = h->n_r_adm_pair, n_node = h->n_node;
    h->n_B = n_pair;
    h->B_nrow = (int *)std::malloc(sizeof(int) * std::max(n_pair, 1));
    h->B_ncol = (int *)std::malloc(sizeof(int) * std::max(n_pair, 1));
    h->B_ptr = (size_t *)std::malloc(sizeof(size_t) * (n_pair + 1));
    h->node_n_r_adm = (int *)std::calloc(n_node, sizeof(int));
    std::vector<int> pi, pj, pv;
    for (int i = 0; i < n_pair; i++) {
        int n0 = h->r_adm_pairs[2 * i], n1 = h->r_adm_pairs[2 * i + 1];
        int l0 = h->node_level[n0], l1 = h->node_level[n1];
        h->node_n_r_adm[n0]++;
        h->node_n_r_adm[n1]++;
        auto leaf_nbfp = [&](int n) {
            return h->sp_bfp_sidx[h->pt_cluster[2 * n + 1] + 1] - h->sp_bfp_sidx[h->pt_cluster[2 * n]];
        };
        h->B_nrow[i] = (l0 >= l1) ? h->J_row[n0]->length : leaf_nbfp(n0);
        h->B_ncol[i] = (l0 <= l1) ? h->J_row[n1]->length : leaf_nbfp(n1);
        pi.push_back(n0); pj.push_back(n1); pv.push_back(i + 1);
        pi.push_back(n1); pj.push_back(n0); pv.push_back(-(i + 1));
    }
    h->B_p2i_rowptr = (int *)std::malloc(sizeof(int) * (n_node + 1));
    h->B_p2i_colidx = (int *)std::malloc(sizeof(int) * std::max<size_t>(pi.size(), 1));
    h->B_p2i_val = (int *)std::malloc(sizeof(int) * std::max<size_t>(pi.size(), 1));
    coo_to_csr(n_node, (int)pi.size(), pi.data(), pj.data(), pv.data(), h->B_p2i_rowptr, h->B_p2i_colidx, h->B_p2i_val);

    h->c_B_blks = (H2E_dense_mat_p *)std::calloc(std::max(n_pair, 1), sizeof(H2E_dense_mat_p));
    /* bra / ket shell pairs of block i and the selected rows / columns */
    auto lists = [&](int i, std::vector<int> &bra, std::vector<int> &ket, const int *&srow, const int *&scol) {
        int n0 = h->r_adm_pairs[2 * i], n1 = h->r_adm_pairs[2 * i + 1];
        int l0 = h->node_level[n0], l1 = h->node_level[n1];
        srow = scol = nullptr;
        if (l0 >= l1) {
            bra.assign(h->J_pair[n0]->data, h->J_pair[n0]->data + h->J_pair[n0]->length);
            srow = h->J_row[n0]->data;
        } else {
            for (int k = h->pt_cluster[2 * n0]; k <= h->pt_cluster[2 * n0 + 1]; k++) bra.push_back(h->index_seq[k]);
        }
        if (l0 <= l1) {
            ket.assign(h->J_pair[n1]->data, h->J_pair[n1]->data + h->J_pair[n1]->length);
            scol = h->J_row[n1]->data;
        } else {
            for (int k = h->pt_cluster[2 * n1]; k <= h->pt_cluster[2 * n1 + 1]; k++) ket.push_back(h->index_seq[k]);
        }
    };
    int done = 0;
    if (EriSet *es = setup_eri(h)) {
        /* full blocks on the GPU in groups of at most 2^27 doubles, rows and
         * columns selected and blocks compressed on the host, the next group
         * evaluated meanwhile */
        std::vector<int> gstart(1, 0);
        long long tot = 0;
        for (int i = 0; i < n_pair; i++) {
            std::vector<int> bra, ket;
            const int *sr, *sc;
            lists(i, bra, ket, sr, sc);
            const long long n = (long long)sum_nbfp(h, bra.data(), (int)bra.size()) *
                                sum_nbfp(h, ket.data(), (int)ket.size());
            if (i > gstart.back() && tot + n > (gstart.size() == 1 ? (1LL << 25) : (1LL << 27))) {
                gstart.push_back(i);
                tot = 0;
            }
            tot += n;
        }
        gstart.push_back(n_pair);
        const int n_groups = (int)gstart.size() - 1;
        std::vector<std::vector<std::vector<double>>> full(2);
        auto prep = [&](int g, std::vector<EriReq> &reqs) {
            std::vector<std::vector<double>> &f = full[g & 1];
            f.clear();
            for (int i = gstart[g]; i < gstart[g + 1]; i++) {
                EriReq q;
                const int *sr, *sc;
                lists(i, q.bra, q.ket, sr, sc);
                const int fc = sum_nbfp(h, q.ket.data(), (int)q.ket.size());
                f.emplace_back((size_t)sum_nbfp(h, q.bra.data(), (int)q.bra.size()) * fc);
                q.ld = fc;
                reqs.push_back(std::move(q));
            }
            for (size_t k = 0; k < reqs.size(); k++) reqs[k].out = f[k].data();
        };
        auto use = [&](int g, std::vector<EriReq> &reqs) {
            std::vector<std::vector<double>> &f = full[g & 1];
            #pragma omp parallel for schedule(dynamic, 1)
            for (int k = 0; k < (int)reqs.size(); k++) {
                const int i = gstart[g] + k;
                std::vector<int> bra, ket;
                const int *srow, *scol;
                lists(i, bra, ket, srow, scol);
                H2E_dense_mat_p blk = dmat_new(h->B_nrow[i], h->B_ncol[i]);
                const int fc = reqs[k].ld;
                for (int r = 0; r < blk->nrow; r++) {
                    const double *src = f[k].data() + (size_t)(srow ? srow[r] : r) * fc;
                    double *dst = blk->data + (size_t)r * blk->ncol;
                    for (int c = 0; c < blk->ncol; c++) dst[c] = src[scol ? scol[c] : c];
                }
                h->c_B_blks[i] = compress_block(blk, h->QR_stop_tol);
                dmat_free(&blk);
            }
            f.clear();
        };
        auto discard = [&](int g, std::vector<EriReq> &) { full[g & 1].clear(); };
        const int used = gpu_pipeline<EriReq>(
            h, n_groups, [es](std::vector<EriReq> &r) { return gpu_eri_blocks(es, r); }, prep, use, discard);
        done = gstart[used];
    }
    #pragma omp parallel for schedule(dynamic, 1)
    for (int i = done; i < n_pair; i++) {
        std::vector<int> bra, ket;
        const int *srow = nullptr, *scol = nullptr;
        lists(i, bra, ket, srow, scol);
        H2E_dense_mat_p blk = dmat_new(h->B_nrow[i], h->B_ncol[i]);
        eri_block(h, bra.data(), (int)bra.size(), ket.data(), (int)ket.size(), srow, h->B_nrow[i], scol,
                  h->B_ncol[i], blk->data);
        h->c_B_blks[i] = compress_block(blk, h->QR_stop_tol);
        dmat_free(&blk);
    }
    h->mat_size[MV_MID_SIZE_IDX] = 0;
    h->B_ptr[0] = 0;
    size_t total = 0;
    std::vector<size_t> sizes(std::max(n_pair, 1));
    for (int i = 0; i < n_pair; i++) {
        size_t s = (size_t)h->c_B_blks[i]->size;
        h->mat_size[MV_MID_SIZE_IDX] += s + 2 * (size_t)(h->B_nrow[i] + h->B_ncol[i]);
        sizes[i] = s;
        total += s;
        h->B_ptr[i + 1] = h->B_ptr[i] + s;
    }
    partition_workload(n_pair, sizes.data(), total, h->n_thread, h->B_blk);
    h->mat_size[B_SIZE_IDX] = total;
}

/* Near-field blocks (src/H2ERI_build_H2.c:1159-1403). Diagonal blocks are
 * symmetric; only their upper shell-pair triangle is evaluated and mirrored. */
void build_D(H2ERI_p h)
{
    const int n_leaf = h->n_leaf_node, n_pair = h->n_r_inadm_pair, n_node = h->n_node;
    const int n_D = n_leaf + n_pair;
    h->n_D = n_D;
    h->D_nrow = (int *)std::malloc(sizeof(int) * std::max(n_D, 1));
    h->D_ncol = (int *)std::malloc(sizeof(int) * std::max(n_D, 1));
    h->D_ptr = (size_t *)std::malloc(sizeof(size_t) * (n_D + 1));
    auto leaf_nbfp = [&](int n) {
        return h->sp_bfp_sidx[h->pt_cluster[2 * n + 1] + 1] - h->sp_bfp_sidx[h->pt_cluster[2 * n]];
    };
    std::vector<int> pi, pj, pv;
    for (int i = 0; i < n_leaf; i++) {
        int node = h->height_nodes[i];
        h->D_nrow[i] = h->D_ncol[i] = leaf_nbfp(node);
        pi.push_back(node); pj.push_back(node); pv.push_back(i + 1);
    }
    for (int i = 0; i < n_pair; i++) {
        int n0 = h->r_inadm_pairs[2 * i], n1 = h->r_inadm_pairs[2 * i + 1];
        h->D_nrow[n_leaf + i] = leaf_nbfp(n0);
        h->D_ncol[n_leaf + i] = leaf_nbfp(n1);
        pi.push_back(n0); pj.push_back(n1); pv.push_back(n_leaf + i + 1);
        pi.push_back(n1); pj.push_back(n0); pv.push_back(-(n_leaf + i + 1));
    }
    h->D_p2i_rowptr = (int *)std::malloc(sizeof(int) * (n_node + 1));
    h->D_p2i_colidx = (int *)std::malloc(sizeof(int) * std::max<size_t>(pi.size(), 1));
    h->D_p2i_val = (int *)std::malloc(sizeof(int) * std::max<size_t>(pi.size(), 1));
    coo_to_csr(n_node, (int)pi.size(), pi.data(), pj.data(), pv.data(), h->D_p2i_rowptr, h->D_p2i_colidx, h->D_p2i_val);

    h->c_D_blks = (H2E_dense_mat_p *)std::calloc(std::max(n_D, 1), sizeof(H2E_dense_mat_p));
    /* larger blocks first for load balance */
    std::vector<int> order(n_D);
    for (int i = 0; i < n_D; i++) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        return (size_t)h->D_nrow[a] * h->D_ncol[a] > (size_t)h->D_nrow[b] * h->D_ncol[b];
    });
    int done = 0;
    if (EriSet *es = setup_eri(h)) {
        /* dense blocks on the GPU in groups of at most 2^27 doubles, each group
         * compressed on the host while the next is evaluated */
        std::vector<int> gstart(1, 0);
        long long tot = 0;
        for (int t = 0; t < n_D; t++) {
            const long long n = (long long)h->D_nrow[order[t]] * h->D_ncol[order[t]];
            if (t > gstart.back() && tot + n > (gstart.size() == 1 ? (1LL << 25) : (1LL << 27))) {
                gstart.push_back(t);
                tot = 0;
            }
            tot += n;
        }
        gstart.push_back(n_D);
        const int n_groups = (int)gstart.size() - 1;
        std::vector<std::vector<H2E_dense_mat_p>> blks(2);
        auto prep = [&](int g, std::vector<EriReq> &reqs) {
            std::vector<H2E_dense_mat_p> &b = blks[g & 1];
            b.clear();
            for (int t = gstart[g]; t < gstart[g + 1]; t++) {
                const int i = order[t];
                EriReq q;
                d_block_lists(h, i, q.bra, q.ket, q.sym);
                b.push_back(dmat_new(h->D_nrow[i], h->D_ncol[i]));
                q.out = b.back()->data;
                q.ld = b.back()->ncol;
                reqs.push_back(std::move(q));
            }
        };
        auto use = [&](int g, std::vector<EriReq> &) {
            std::vector<H2E_dense_mat_p> &b = blks[g & 1];
            #pragma omp parallel for schedule(dynamic, 1)
            for (int k = 0; k < (int)b.size(); k++) {
                h->c_D_blks[order[gstart[g] + k]] = compress_block(b[k], h->QR_stop_tol);
                dmat_free(&b[k]);
            }
            b.clear();
        };
        auto discard = [&](int g, std::vector<EriReq> &) {
            for (H2E_dense_mat_p &x : blks[g & 1]) dmat_free(&x);
            blks[g & 1].clear();
        };
        const int used = gpu_pipeline<EriReq>(
            h, n_groups, [es](std::vector<EriReq> &r) { return gpu_eri_blocks(es, r); }, prep, use, discard);
        done = gstart[used];
    }
    const double th = wtime();
    #pragma omp parallel for schedule(dynamic, 1)
    for (int t = done; t < n_D; t++) {
        int i = order[t];
        H2E_dense_mat_p blk = dmat_new(h->D_nrow[i], h->D_ncol[i]);
        d_block_host(h, i, blk);
        h->c_D_blks[i] = compress_block(blk, h->QR_stop_tol);
        dmat_free(&blk);
    }
    if (setup_verbose() && done < n_D)
        std::fprintf(stderr, "build_D: %d blocks on the host engine (integrals and compression) %.3f s\n", n_D - done,
                     wtime() - th);
    h->mat_size[MV_DEN_SIZE_IDX] = 0;
    h->D_ptr[0] = 0;
    std::vector<size_t> sizes(std::max(n_D, 1));
    size_t tot0 = 0, tot1 = 0;
    for (int i = 0; i < n_D; i++) {
        H2E_dense_mat_p d = h->c_D_blks[i];
        size_t s = (size_t)d->size;
        sizes[i] = s;
        h->mat_size[MV_DEN_SIZE_IDX] += s + (size_t)(d->nrow + d->ncol) * (i < n_leaf ? 1 : 2);
        if (i < n_leaf) tot0 += s; else tot1 += s;
        h->D_ptr[i + 1] = h->D_ptr[i] + s;
    }
    partition_workload(n_leaf, sizes.data(), tot0, h->n_thread, h->D_blk0);
    partition_workload(n_pair, sizes.data() + n_leaf, tot1, h->n_thread, h->D_blk1);
    h->mat_size[D_SIZE_IDX] = tot0 + tot1;
}

}  // namespace

void build_h2(H2ERI_p h)
{
    double t0 = wtime();
    build_UJ_proxy(h);
    double t1 = wtime();
    build_B(h);
    double t2 = wtime();
    build_D(h);
    setup_eri_end();
    double t3 = wtime();
    h->timers[U_BUILD_TIMER_IDX] = t1 - t0;
    h->timers[B_BUILD_TIMER_IDX] = t2 - t1;
    h->timers[D_BUILD_TIMER_IDX] = t3 - t2;
}

}  // namespace h2g

extern "C" int h2g_id_rows(int nrow, int ncol, const double *A, double rel_tol, int *J, double *U)
{
    using namespace h2g;
    H2E_dense_mat_p M = dmat_new(nrow, ncol);
    if ((size_t)nrow * ncol > 0) std::memcpy(M->data, A, sizeof(double) * (size_t)nrow * ncol);
    H2E_int_vec_p Jv = ivec_new(std::max(nrow, 1));
    H2E_dense_mat_p Um = nullptr;
    id_compress(M, rel_tol, &Um, Jv);
    const int r = Jv->length;
    std::memcpy(J, Jv->data, sizeof(int) * (size_t)r);
    if (r > 0) std::memcpy(U, Um->data, sizeof(double) * (size_t)nrow * r);
    dmat_free(&M);
    dmat_free(&Um);
    ivec_free(&Jv);
    return r;
}

/* Dense near-field blocks and full coupling blocks (before compression) of
 * a built structure from the GPU engine and from the host engine: up to
 * max_blocks of each kind (diagonal near-field, inadmissible near-field,
 * coupling). out: [0] largest |difference|, [1] largest |value|, [2]
 * elements compared, [3] blocks compared, [4] seconds of the GPU evaluation
 * (with the copy back), [5] seconds of the host engine (one thread, with the
 * host-side bookkeeping of the check). Returns 0, or an error code (no
 * usable device: 9). */
extern "C" int H2ERI_gpu_setup_eri_check(H2ERI_p h, int max_blocks, double *out)
{
    using namespace h2g;
    if (h == nullptr || out == nullptr || max_blocks < 1) return 3;
    if (!gpu_eri_usable()) return 9;
    std::vector<const h2g_pair *> pairs(h->num_sp);
    for (int i = 0; i < h->num_sp; i++) pairs[i] = sp_pair(h, i);
    EriSet *es = nullptr;
    int rc = gpu_eri_create(h->num_sp, pairs.data(), &es);
    if (rc) return rc;
    std::vector<EriReq> reqs;
    std::vector<std::vector<double>> ref;
    const int n_leaf = h->n_leaf_node, n_D = h->n_D;
    auto add_d = [&](int i) {
        EriReq q;
        d_block_lists(h, i, q.bra, q.ket, q.sym);
        H2E_dense_mat_p blk = dmat_new(h->D_nrow[i], h->D_ncol[i]);
        d_block_host(h, i, blk);
        ref.emplace_back(blk->data, blk->data + (size_t)blk->nrow * blk->ncol);
        q.ld = blk->ncol;
        dmat_free(&blk);
        reqs.push_back(std::move(q));
    };
    double t_host = 0.0;
    const double th0 = wtime();
    for (int i = 0; i < std::min(max_blocks, n_leaf); i++) add_d(i);
    for (int i = n_leaf; i < std::min(n_D, n_leaf + max_blocks); i++) add_d(i);
    for (int i = 0; i < std::min(max_blocks, h->n_r_adm_pair); i++) {
        EriReq q;
        int n0 = h->r_adm_pairs[2 * i], n1 = h->r_adm_pairs[2 * i + 1];
        int l0 = h->node_level[n0], l1 = h->node_level[n1];
        if (l0 >= l1) q.bra.assign(h->J_pair[n0]->data, h->J_pair[n0]->data + h->J_pair[n0]->length);
        else for (int k = h->pt_cluster[2 * n0]; k <= h->pt_cluster[2 * n0 + 1]; k++) q.bra.push_back(h->index_seq[k]);
        if (l0 <= l1) q.ket.assign(h->J_pair[n1]->data, h->J_pair[n1]->data + h->J_pair[n1]->length);
        else for (int k = h->pt_cluster[2 * n1]; k <= h->pt_cluster[2 * n1 + 1]; k++) q.ket.push_back(h->index_seq[k]);
        const int fr = sum_nbfp(h, q.bra.data(), (int)q.bra.size()), fc = sum_nbfp(h, q.ket.data(), (int)q.ket.size());
        std::vector<double> full((size_t)fr * fc);
        eri_pairs_to_mat(h, (int)q.bra.size(), q.bra.data(), (int)q.ket.size(), q.ket.data(), full.data(), fc);
        ref.push_back(std::move(full));
        q.ld = fc;
        reqs.push_back(std::move(q));
    }
    t_host = wtime() - th0;
    std::vector<std::vector<double>> got(reqs.size());
    for (size_t k = 0; k < reqs.size(); k++) {
        got[k].assign(ref[k].size(), std::nan(""));
        reqs[k].out = got[k].data();
    }
    const double tg0 = wtime();
    rc = gpu_eri_blocks(es, reqs);
    const double t_gpu = wtime() - tg0;
    gpu_eri_free(es);
    if (rc) return rc;
    double dmax = 0.0, vmax = 0.0, n = 0.0;
    for (size_t k = 0; k < reqs.size(); k++)
        for (size_t e = 0; e < ref[k].size(); e++) {
            const double d = std::fabs(got[k][e] - ref[k][e]);
            dmax = std::isnan(d) ? INFINITY : std::max(dmax, d);
            vmax = std::max(vmax, std::fabs(ref[k][e]));
            n += 1.0;
        }
    out[0] = dmax;
    out[1] = vmax;
    out[2] = n;
    out[3] = (double)reqs.size();
    out[4] = t_gpu;
    out[5] = t_host;
    return 0;
}

/* The sketched integral matrices of the nested-basis set-up (proxy-point
 * potentials and far-field ERIs, each times its sparse sign sketch) of up to
 * max_nodes nodes of a built structure, from the GPU and from the host
 * engine, on the same inputs: nodes taken level by level from the leaves,
 * every far-field shell pair counted as a skeleton. out: [0] largest
 * |difference|, [1] largest |value|, [2] elements compared, [3] nodes
 * compared, [4] seconds on the GPU (with the copy back), [5] seconds of the
 * host engine (one thread). Returns 0, or an error code (no usable device:
 * 9). */
extern "C" int H2ERI_gpu_setup_u_check(H2ERI_p h, int max_nodes, double *out)
{
    using namespace h2g;
    if (h == nullptr || out == nullptr || max_nodes < 1) return 3;
    if (h->ovlp_ff_idx == nullptr || h->J_pair == nullptr) return 3;
    if (!gpu_eri_usable()) return 9;
    std::vector<const h2g_pair *> pairs(h->num_sp);
    for (int i = 0; i < h->num_sp; i++) pairs[i] = sp_pair(h, i);
    EriSet *es = nullptr;
    int rc = gpu_eri_create(h->num_sp, pairs.data(), &es);
    if (rc) return rc;
    std::vector<int> skel(h->n_point, 1), nodes;
    for (int lv = h->max_level; lv >= h->min_adm_level && (int)nodes.size() < max_nodes; lv--)
        for (int j = 0; j < h->level_n_node[lv] && (int)nodes.size() < max_nodes; j++)
            nodes.push_back(h->level_nodes[lv * h->n_leaf_node + j]);
    std::vector<UNode> W(nodes.size());
    std::vector<std::vector<double>> ref(nodes.size());
    double t_nai = 0.0, t_eri = 0.0;
    for (size_t k = 0; k < nodes.size(); k++) {
        u_prep(h, nodes[k], skel, W[k]);
        u_integrals_host(h, W[k], t_nai, t_eri);
        ref[k] = W[k].A;
        std::fill(W[k].A.begin(), W[k].A.end(), std::nan(""));
    }
    std::vector<UReq> reqs;
    for (UNode &w : W)
        if (w.nrow_blk > 0) reqs.push_back(u_request(w));
    const double tg0 = wtime();
    rc = gpu_u_blocks(es, reqs);
    const double t_gpu = wtime() - tg0;
    gpu_eri_free(es);
    if (rc) return rc;
    double dmax = 0.0, vmax = 0.0, n = 0.0;
    for (size_t k = 0; k < W.size(); k++)
        for (size_t e = 0; e < ref[k].size(); e++) {
            const double d = std::fabs(W[k].A[e] - ref[k][e]);
            dmax = std::isnan(d) ? INFINITY : std::max(dmax, d);
            vmax = std::max(vmax, std::fabs(ref[k][e]));
            n += 1.0;
        }
    out[0] = dmax;
    out[1] = vmax;
    out[2] = n;
    out[3] = (double)reqs.size();
    out[4] = t_gpu;
    out[5] = t_nai + t_eri;
    return 0;
}

extern "C" void H2ERI_build_H2(H2ERI_p h2eri, const int BD_JIT)
{
    H2G_CHECK(BD_JIT == 0,
              "H2ERI_build_H2: BD_JIT=1 (just-in-time B/D) is not supported; the GPU hot path needs the "
              "blocks built ahead of time\n");
    H2G_CHECK(h2eri->n_node > 0, "H2ERI_build_H2: call H2ERI_partition first\n");
    h2eri->BD_JIT = 0;
    h2g::build_h2(h2eri);
}
