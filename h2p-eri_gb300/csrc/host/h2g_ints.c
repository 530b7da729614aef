/*
 * Gaussian integral engine: ERI (Obara-Saika VRR + Head-Gordon-Pople HRR) and
 * point-charge potential integrals, plus the Boys function. See h2g_ints.h for
 * the conventions (they follow what the reference expects from SIMINT:
 * H2P-ERI src/CMS.c:387-482, src/H2ERI_partition.c:84-96).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#include "h2g_ints.h"

#define H2G_MAX_L    (2 * H2G_MAX_AM)          /* max total L on one side */
#define H2G_MAX_M    (4 * H2G_MAX_AM + 1)      /* max Boys order used     */
#define H2G_NCUM(L)  (((L) + 1) * ((L) + 2) * ((L) + 3) / 6)
#define H2G_MAXCUM   H2G_NCUM(H2G_MAX_L)

/* ------------------------------------------------------------------------ */
/* Cartesian component tables                                               */
/* ------------------------------------------------------------------------ */

/* Flat index over all components with total L <= H2G_MAX_L, ordered by L then
 * by the standard in-shell order. */
static int g_lxyz[H2G_MAXCUM][3];
static int g_cum[H2G_MAX_L + 2];             /* first flat index of each L     */
static int g_dir[H2G_MAXCUM];                /* recurrence direction          */
static int g_prev[H2G_MAXCUM];               /* c - 1_dir                      */
static int g_prev2[H2G_MAXCUM];              /* c - 2_dir (or -1)              */
static int g_minus[H2G_MAXCUM][3];           /* c - 1_i (or -1)                */
static int g_plus[H2G_MAXCUM][3];            /* c + 1_i (or -1 beyond table)   */

static int flat_index(int lx, int ly, int lz)
{
    int L = lx + ly + lz;
    /* position inside shell L: components ordered by decreasing lx, then ly */
    int pos = 0;
    for (int x = L; x > lx; x--) pos += L - x + 1;
    pos += (L - lx) - ly;
    return g_cum[L] + pos;
}

/* ------------------------------------------------------------------------ */
/* Boys function table                                                      */
/* ------------------------------------------------------------------------ */

#define BOYS_H      0.05
#define BOYS_TMAX   40.0
#define BOYS_NGRID  801                 /* 0 .. 40 step 0.05 */
#define BOYS_NTAY   7
#define BOYS_MTAB   (H2G_MAX_M + BOYS_NTAY + 1)

static double g_boys_tab[BOYS_NGRID][BOYS_MTAB];
static pthread_once_t g_once = PTHREAD_ONCE_INIT;

/* F_m(T) = exp(-T) sum_i (2T)^i / ((2m+1)(2m+3)...(2m+2i+1)), evaluated in
 * long double; converges for every T (terms peak near i ~ T). */
static long double boys_series(int m, long double T)
{
    long double term = 1.0L / (2 * m + 1), sum = term;
    for (int i = 1; i < 2000; i++) {
        term *= 2.0L * T / (long double)(2 * m + 2 * i + 1);
        sum += term;
        if (term < sum * 1e-21L) break;
    }
    return expl(-T) * sum;
}

static void init_tables(void)
{
    int idx = 0;
    for (int L = 0; L <= H2G_MAX_L; L++) {
        g_cum[L] = idx;
        for (int lx = L; lx >= 0; lx--)
            for (int ly = L - lx; ly >= 0; ly--) {
                g_lxyz[idx][0] = lx; g_lxyz[idx][1] = ly; g_lxyz[idx][2] = L - lx - ly;
                idx++;
            }
    }
    g_cum[H2G_MAX_L + 1] = idx;
    for (int c = 0; c < idx; c++) {
        const int *l = g_lxyz[c];
        for (int i = 0; i < 3; i++) {
            int t[3] = {l[0], l[1], l[2]};
            t[i]--;
            g_minus[c][i] = (t[i] >= 0) ? flat_index(t[0], t[1], t[2]) : -1;
            t[i] += 2;
            g_plus[c][i] = (t[0] + t[1] + t[2] <= H2G_MAX_L) ? flat_index(t[0], t[1], t[2]) : -1;
        }
        if (c == 0) { g_dir[c] = -1; g_prev[c] = -1; g_prev2[c] = -1; continue; }
        int d = (l[0] > 0) ? 0 : ((l[1] > 0) ? 1 : 2);
        g_dir[c] = d;
        g_prev[c] = g_minus[c][d];
        g_prev2[c] = (l[d] >= 2) ? g_minus[g_prev[c]][d] : -1;
    }
    for (int k = 0; k < BOYS_NGRID; k++) {
        long double T = (long double)k * BOYS_H;
        for (int m = 0; m < BOYS_MTAB; m++) g_boys_tab[k][m] = (double)boys_series(m, T);
    }
}

void h2g_ints_init(void) { pthread_once(&g_once, init_tables); }

int h2g_ints_tables(int *lxyz, int *cum, int *dir, int *prev, int *prev2, int *minus, int *plus, double *boys,
                    int *dims)
{
    h2g_ints_init();
    dims[0] = H2G_MAX_L;
    dims[1] = H2G_MAXCUM;
    dims[2] = BOYS_NGRID;
    dims[3] = BOYS_MTAB;
    if (lxyz) memcpy(lxyz, g_lxyz, sizeof(g_lxyz));
    if (cum) memcpy(cum, g_cum, sizeof(g_cum));
    if (dir) memcpy(dir, g_dir, sizeof(g_dir));
    if (prev) memcpy(prev, g_prev, sizeof(g_prev));
    if (prev2) memcpy(prev2, g_prev2, sizeof(g_prev2));
    if (minus) memcpy(minus, g_minus, sizeof(g_minus));
    if (plus) memcpy(plus, g_plus, sizeof(g_plus));
    if (boys) memcpy(boys, g_boys_tab, sizeof(g_boys_tab));
    return 0;
}

void h2g_boys(int mmax, double T, double *F)
{
    if (T < BOYS_TMAX) {
        int k = (int)(T / BOYS_H + 0.5);
        double d = T - k * BOYS_H;                   /* |d| <= h/2 */
        const double *row = g_boys_tab[k];
        /* F_m(T_k + d) = sum_j F_{m+j}(T_k) (-d)^j / j!, the factors shared by all m */
        _Static_assert(BOYS_NTAY == 7, "one factor 1/j! per Taylor term");
        static const double inv_fact[BOYS_NTAY] = {1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720};
        double f[BOYS_NTAY], pw = 1.0;
        for (int j = 0; j < BOYS_NTAY; j++) {
            f[j] = pw * inv_fact[j];
            pw *= -d;
        }
        for (int m = 0; m <= mmax; m++) {
            double s = 0.0;
            for (int j = 0; j < BOYS_NTAY; j++) s += row[m + j] * f[j];
            F[m] = s;
        }
    } else {
        double et = exp(-T), inv2t = 0.5 / T;
        F[0] = 0.5 * sqrt(M_PI / T);                  /* erf(sqrt(T)) == 1 here */
        for (int m = 0; m < mmax; m++) F[m + 1] = ((2 * m + 1) * F[m] - et) * inv2t;
    }
}

/* ------------------------------------------------------------------------ */
/* Shell normalisation                                                      */
/* ------------------------------------------------------------------------ */

static double dfact_odd(int L) /* (2L-1)!! with (-1)!! = 1 */
{
    double r = 1.0;
    for (int k = 2 * L - 1; k > 1; k -= 2) r *= k;
    return r;
}

void h2g_normalize_shell(int am, int nprim, const double *alpha, double *coef)
{
    const double m = am + 1.5, m2 = 0.5 * m;
    double sum = 0.0;
    for (int j = 0; j < nprim; j++)
        for (int k = 0; k < nprim; k++)
            sum += coef[j] * coef[k] * pow(alpha[j] * alpha[k], m2) / pow(alpha[j] + alpha[k], m);
    /* <x^L g_j | x^L g_k> for raw Gaussians = pi^1.5 (2L-1)!! / (2^L (a_j+a_k)^(L+1.5)) */
    double fac = pow(M_PI, 1.5) * dfact_odd(am) / pow(2.0, am);
    double norm = 1.0 / sqrt(sum * fac);
    for (int j = 0; j < nprim; j++) coef[j] *= norm * pow(alpha[j], m2);
}

/* ------------------------------------------------------------------------ */
/* Primitive-pair data                                                      */
/* ------------------------------------------------------------------------ */

void h2g_pair_init(h2g_pair *pr, const h2g_shell *A, const h2g_shell *B)
{
    h2g_ints_init();
    pr->am1 = A->am; pr->am2 = B->am;
    pr->A[0] = A->x; pr->A[1] = A->y; pr->A[2] = A->z;
    pr->B[0] = B->x; pr->B[1] = B->y; pr->B[2] = B->z;
    int np = A->nprim * B->nprim;
    pr->P = (double *)malloc(sizeof(double) * (size_t)np * 3);
    pr->p = (double *)malloc(sizeof(double) * (size_t)np);
    pr->K = (double *)malloc(sizeof(double) * (size_t)np);
    pr->ip = (double *)malloc(sizeof(double) * (size_t)np);
    double ab2 = 0.0;
    for (int d = 0; d < 3; d++) ab2 += (pr->A[d] - pr->B[d]) * (pr->A[d] - pr->B[d]);
    int n = 0;
    for (int i = 0; i < A->nprim; i++)
        for (int j = 0; j < B->nprim; j++) {
            double a = A->alpha[i], b = B->alpha[j], p = a + b;
            double K = A->coef[i] * B->coef[j] * exp(-a * b / p * ab2);
            if (fabs(K) < 1e-30) continue;
            pr->p[n] = p;
            pr->K[n] = K;
            pr->ip[n] = 1.0 / p;
            for (int d = 0; d < 3; d++) pr->P[3 * n + d] = (a * pr->A[d] + b * pr->B[d]) / p;
            n++;
        }
    pr->nprim = n;
}

void h2g_pair_free(h2g_pair *pr)
{
    free(pr->P); free(pr->p); free(pr->K); free(pr->ip);
    pr->P = pr->p = pr->K = pr->ip = NULL;
    pr->nprim = 0;
}

/* ------------------------------------------------------------------------ */
/* Horizontal recurrence                                                    */
/* ------------------------------------------------------------------------ */

/* Transfer angular momentum from the first to the second index of a pair:
 *   (a, b + 1_i| = (a + 1_i, b| + AB_i (a, b|
 * in:  src[e * stride] for flat e with l1 <= |e| <= l1 + l2 (flat cumulative
 *      index), repeated over `nrep` independent trailing entries (stride apart
 *      handled by caller through `nrep` contiguous values per e).
 * out: dst[(ia * nb + ib) * nrep + r] with ia over comps of l1, ib over l2. */
static void hrr(int l1, int l2, const double AB[3], const double *src, int nrep, double *dst, double *work)
{
    const int na = h2g_ncart(l1), nb = h2g_ncart(l2);
    if (l2 == 0) {
        memcpy(dst, src + (size_t)g_cum[l1] * nrep, sizeof(double) * (size_t)na * nrep);
        return;
    }
    /* cur[e][b][r]: e flat over cumulative index, b within shell of current level j */
    const int ne = g_cum[l1 + l2 + 1];
    double *cur = work, *nxt = work + (size_t)ne * h2g_ncart(l2) * nrep;
    /* level 0: b = s */
    for (int e = g_cum[l1]; e < ne; e++)
        memcpy(cur + (size_t)e * nrep, src + (size_t)e * nrep, sizeof(double) * nrep);
    for (int j = 1; j <= l2; j++) {
        int nbj = h2g_ncart(j), nbp = h2g_ncart(j - 1);
        int emax = g_cum[l1 + l2 - j + 1];
        for (int e = g_cum[l1]; e < emax; e++) {
            for (int ib = 0; ib < nbj; ib++) {
                int bf = g_cum[j] + ib;
                int d = g_dir[bf];
                int bp = g_prev[bf] - g_cum[j - 1];
                int ep = g_plus[e][d];
                const double *x1 = cur + ((size_t)ep * nbp + bp) * nrep;
                const double *x2 = cur + ((size_t)e * nbp + bp) * nrep;
                double *y = nxt + ((size_t)e * nbj + ib) * nrep;
                double ab = AB[d];
                for (int r = 0; r < nrep; r++) y[r] = x1[r] + ab * x2[r];
            }
        }
        double *t = cur; cur = nxt; nxt = t;
    }
    for (int ia = 0; ia < na; ia++)
        memcpy(dst + (size_t)ia * nb * nrep, cur + (size_t)(g_cum[l1] + ia) * nb * nrep,
               sizeof(double) * (size_t)nb * nrep);
}

/* ------------------------------------------------------------------------ */
/* ERI                                                                      */
/* ------------------------------------------------------------------------ */

/* Primitive quartets are processed H2G_LANES at a time: every recurrence
 * term is a GCC vector of one value per quartet (element-wise IEEE
 * arithmetic, no instruction-set header), so the index bookkeeping of the
 * recurrences is shared by the lanes. */
#define H2G_LANES 4
typedef double vlane __attribute__((vector_size(H2G_LANES * sizeof(double))));
_Static_assert(H2G_LANES == 4, "the lane sums below add four lanes");

typedef struct {
    vlane *vrr;       /* [(e nf + f) nm + m], grown to the largest class seen */
    size_t vrr_cap;
    double acc[H2G_NCUM(H2G_MAX_L) * H2G_NCUM(H2G_MAX_L)];
    double t1[H2G_NCUM(H2G_MAX_L) * H2G_NCUM(H2G_MAX_L) * 8];
    double w1[2 * H2G_NCUM(H2G_MAX_L) * H2G_NCUM(H2G_MAX_L) * 16];
} eri_ws;

static __thread eri_ws *tls_ws = NULL;

static eri_ws *get_ws(void)
{
    if (tls_ws == NULL) {
        tls_ws = (eri_ws *)malloc(sizeof(eri_ws));
        tls_ws->vrr = NULL;
        tls_ws->vrr_cap = 0;
    }
    return tls_ws;
}

static vlane *vrr_buf(eri_ws *ws, size_t n)
{
    if (ws->vrr_cap < n) {
        free(ws->vrr);
        ws->vrr = (vlane *)aligned_alloc(64, ((n * sizeof(vlane) + 63) / 64) * 64);
        ws->vrr_cap = n;
    }
    return ws->vrr;
}

/* Obara-Saika vertical recurrences for one batch of primitive quartets, on
 * values of type T (double, or vlane for H2G_LANES quartets at once):
 * V[(e nf + f) nm + m] = [e|f]^(m), from [0|0]^(m) in V[0..M]. */
#define VRR(T)                                                                                  \
    do {                                                                                        \
        /* bra side: [e|0]^(m) */                                                               \
        for (int c = 1; c < ne; c++) {                                                          \
            const int L = g_lxyz[c][0] + g_lxyz[c][1] + g_lxyz[c][2];                           \
            const int d = g_dir[c], e = g_prev[c], e2 = g_prev2[c];                             \
            T *vc = V + (size_t)c * nf * nm;                                                    \
            const T *ve = V + (size_t)e * nf * nm;                                              \
            if (e2 >= 0) {                                                                      \
                const T *ve2 = V + (size_t)e2 * nf * nm;                                        \
                const T ei2p = (double)(g_lxyz[c][d] - 1) * i2p;                                \
                for (int m = 0; m <= M - L; m++)                                                \
                    vc[m] = PA[d] * ve[m] + WP[d] * ve[m + 1] + ei2p * (ve2[m] - rp * ve2[m + 1]);\
            } else {                                                                            \
                for (int m = 0; m <= M - L; m++) vc[m] = PA[d] * ve[m] + WP[d] * ve[m + 1];     \
            }                                                                                   \
        }                                                                                       \
        /* ket side: [e|f]^(m) */                                                               \
        for (int c = 1; c < nf; c++) {                                                          \
            const int Lf = g_lxyz[c][0] + g_lxyz[c][1] + g_lxyz[c][2];                          \
            const int d = g_dir[c], f = g_prev[c], f2 = g_prev2[c];                             \
            const T fi2q = (double)(g_lxyz[c][d] - 1) * i2q;                                    \
            for (int e = 0; e < ne; e++) {                                                      \
                const int Le = g_lxyz[e][0] + g_lxyz[e][1] + g_lxyz[e][2];                      \
                const int mmax = M - Le - Lf;                                                   \
                if (mmax < 0) continue;                                                         \
                T *vc = V + ((size_t)e * nf + c) * nm;                                          \
                const T *vf = V + ((size_t)e * nf + f) * nm;                                    \
                const T *vf2 = (f2 >= 0) ? V + ((size_t)e * nf + f2) * nm : NULL;               \
                const int em = g_minus[e][d];                                                   \
                const T *vem = (em >= 0) ? V + ((size_t)em * nf + f) * nm : NULL;               \
                const T ed2pq = (double)g_lxyz[e][d] * i2pq;                                    \
                for (int m = 0; m <= mmax; m++) {                                               \
                    T v = QC[d] * vf[m] + WQ[d] * vf[m + 1];                                    \
                    if (vf2) v += fi2q * (vf2[m] - rq * vf2[m + 1]);                            \
                    if (vem) v += ed2pq * vem[m + 1];                                           \
                    vc[m] = v;                                                                  \
                }                                                                               \
            }                                                                                   \
        }                                                                                       \
    } while (0)

void h2g_eri_quartet(const h2g_pair *bra, const h2g_pair *ket, double *out)
{
    const int la = bra->am1, lb = bra->am2, lc = ket->am1, ld = ket->am2;
    const int La = la + lb, Lc = lc + ld, M = La + Lc;
    const int nA = h2g_ncart(la), nB = h2g_ncart(lb), nC = h2g_ncart(lc), nD = h2g_ncart(ld);
    const int ne = g_cum[La + 1], nf = g_cum[Lc + 1], nm = M + 1;
    eri_ws *ws = get_ws();
    double *acc = ws->acc;
    const double two_pi_52 = 2.0 * pow(M_PI, 2.5);

    /* per primitive quartet: 1/(p+q) is the only division; with 1/p and 1/q
     * stored with the primitive pairs,
     *   rho = p q / (p+q), W - P = q (Q - P) / (p+q), W - Q = p (P - Q) / (p+q),
     *   prefactor 2 pi^(5/2) K_ab K_cd / (p q sqrt(p+q)) */
    if (M == 0) {
        double s = 0.0, F[1];
        for (int i = 0; i < bra->nprim; i++) {
            const double p = bra->p[i], *P = bra->P + 3 * i;
            const double kp = two_pi_52 * bra->K[i] / p;
            for (int j = 0; j < ket->nprim; j++) {
                const double q = ket->p[j], *Q = ket->P + 3 * j;
                const double ipq = 1.0 / (p + q), rho = p * q * ipq;
                double dx = P[0] - Q[0], dy = P[1] - Q[1], dz = P[2] - Q[2];
                h2g_boys(0, rho * (dx * dx + dy * dy + dz * dz), F);
                s += kp * (ket->K[j] * ket->ip[j]) * sqrt(ipq) * F[0];
            }
        }
        out[0] = s;
        return;
    }

    memset(acc, 0, sizeof(double) * (size_t)ne * nf);
    if (M == 1) {
        /* one p function in the quartet: [p|s] = PA [s|s]^(0) + WP [s|s]^(1)
         * (or [s|p] = QC [s|s]^(0) + WQ [s|s]^(1)), summed directly */
        const int bra_p = (La == 1);
        const double *C0 = bra_p ? bra->A : ket->A;
        double s0 = 0.0, s1[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < bra->nprim; i++) {
            const double p = bra->p[i], *P = bra->P + 3 * i;
            const double ip = bra->ip[i];
            for (int j = 0; j < ket->nprim; j++) {
                const double q = ket->p[j], *Q = ket->P + 3 * j;
                const double ipq = 1.0 / (p + q), rho = p * q * ipq;
                double pq[3], PQ2 = 0.0;
                for (int d = 0; d < 3; d++) {
                    pq[d] = P[d] - Q[d];
                    PQ2 += pq[d] * pq[d];
                }
                double F[2];
                h2g_boys(1, rho * PQ2, F);
                const double pref = two_pi_52 * bra->K[i] * ip * (ket->K[j] * ket->ip[j]) * sqrt(ipq);
                const double V0 = pref * F[0], V1 = pref * F[1];
                s0 += V0;
                if (bra_p) {
                    const double rp = q * ipq;
                    for (int d = 0; d < 3; d++) s1[d] += (P[d] - C0[d]) * V0 + (-rp * pq[d]) * V1;
                } else {
                    const double rq = p * ipq;
                    for (int d = 0; d < 3; d++) s1[d] += (Q[d] - C0[d]) * V0 + (rq * pq[d]) * V1;
                }
            }
        }
        acc[0] = s0;                               /* [s|s]: ne = 4, nf = 1 or ne = 1, nf = 4 */
        for (int d = 0; d < 3; d++) acc[1 + d] = s1[d];
    }
    vlane *Vv = vrr_buf(ws, (size_t)ne * nf * nm);
    const int nk = ket->nprim, nq = bra->nprim * nk;
    /* one or two primitive quartets: one at a time (lanes would be idle) */
    for (int qi = 0; qi < (M > 1 && nq <= 2 ? nq : 0); qi++) {
        double *V = (double *)Vv;
        const int i = qi / nk, j = qi - i * nk;
        const double p = bra->p[i], *P = bra->P + 3 * i;
        const double q = ket->p[j], *Q = ket->P + 3 * j;
        const double ipq = 1.0 / (p + q), rho = p * q * ipq, ip = bra->ip[i];
        double PA[3], WP[3], WQ[3], QC[3], PQ2 = 0.0;
        for (int d = 0; d < 3; d++) {
            const double pq_d = P[d] - Q[d];
            PA[d] = P[d] - bra->A[d];
            WP[d] = -(q * ipq) * pq_d;
            WQ[d] = (p * ipq) * pq_d;
            QC[d] = Q[d] - ket->A[d];
            PQ2 += pq_d * pq_d;
        }
        const double i2p = 0.5 * ip, rp = q * ipq, i2q = 0.5 * ket->ip[j], rq = p * ipq, i2pq = 0.5 * ipq;
        double F[H2G_MAX_M + 1];
        h2g_boys(M, rho * PQ2, F);
        const double pref = two_pi_52 * bra->K[i] * ip * (ket->K[j] * ket->ip[j]) * sqrt(ipq);
        for (int m = 0; m <= M; m++) V[m] = pref * F[m];
        VRR(double);
        for (int e = g_cum[la]; e < ne; e++)
            for (int f = g_cum[lc]; f < nf; f++) acc[e * nf + f] += V[((size_t)e * nf + f) * nm];
    }
    int ci = 0, cj = 0;   /* (i, j) of primitive quartet q0 */
    for (int q0 = 0; q0 < (M > 1 && nq > 2 ? nq : 0); q0 += H2G_LANES) {
        vlane *V = Vv;
        /* lane l holds primitive quartet q0 + l = (i, j); lanes past the end
         * repeat quartet q0 with a zero prefactor, so they add zeros */
        vlane PA[3], WP[3], WQ[3], QC[3], i2p, rp, i2q, rq, i2pq;
        double F[H2G_LANES][H2G_MAX_M + 1], pref[H2G_LANES];
        const int i0 = ci, j0 = cj;
        for (int l = 0; l < H2G_LANES; l++) {
            const int live = q0 + l < nq;
            const int i = live ? ci : i0, j = live ? cj : j0;
            if (live && ++cj == nk) { cj = 0; ci++; }
            const double p = bra->p[i], *P = bra->P + 3 * i;
            const double q = ket->p[j], *Q = ket->P + 3 * j;
            const double ipq = 1.0 / (p + q), rho = p * q * ipq, ip = bra->ip[i];
            double PQ2 = 0.0;
            for (int d = 0; d < 3; d++) {
                const double pq_d = P[d] - Q[d];
                PA[d][l] = P[d] - bra->A[d];
                WP[d][l] = -(q * ipq) * pq_d;
                WQ[d][l] = (p * ipq) * pq_d;
                QC[d][l] = Q[d] - ket->A[d];
                PQ2 += pq_d * pq_d;
            }
            i2p[l] = 0.5 * ip;
            rp[l] = q * ipq;
            i2q[l] = 0.5 * ket->ip[j];
            rq[l] = p * ipq;
            i2pq[l] = 0.5 * ipq;
            h2g_boys(M, rho * PQ2, F[l]);
            pref[l] = live ? two_pi_52 * bra->K[i] * ip * (ket->K[j] * ket->ip[j]) * sqrt(ipq) : 0.0;
        }
        for (int m = 0; m <= M; m++)
            for (int l = 0; l < H2G_LANES; l++) V[m][l] = pref[l] * F[l][m];
        VRR(vlane);
        for (int e = g_cum[la]; e < ne; e++)
            for (int f = g_cum[lc]; f < nf; f++) {
                const vlane v = V[((size_t)e * nf + f) * nm];
                acc[e * nf + f] += (v[0] + v[1]) + (v[2] + v[3]);   /* H2G_LANES == 4 */
            }
    }

    /* HRR on the bra: acc[e][f] -> t1[(a b)][f], f kept as a trailing vector */
    double ABv[3] = {bra->A[0] - bra->B[0], bra->A[1] - bra->B[1], bra->A[2] - bra->B[2]};
    double CDv[3] = {ket->A[0] - ket->B[0], ket->A[1] - ket->B[1], ket->A[2] - ket->B[2]};
    double *t1 = ws->t1;
    hrr(la, lb, ABv, acc, nf, t1, ws->w1);
    /* HRR on the ket for each (a,b) */
    const int nab = nA * nB;
    for (int ab = 0; ab < nab; ab++)
        hrr(lc, ld, CDv, t1 + (size_t)ab * nf, 1, out + (size_t)ab * nC * nD, ws->w1);
}

/* ------------------------------------------------------------------------ */
/* Point-charge potential integrals                                         */
/* ------------------------------------------------------------------------ */

void h2g_potential_points(const h2g_shell *A, const h2g_shell *B, int n_pt, const double *cx,
                          const double *cy, const double *cz, double charge, double *out, int ldo)
{
    h2g_ints_init();
    const int la = A->am, lb = B->am, L = la + lb;
    const int ne = g_cum[L + 1], nm = L + 1, nab = h2g_ncart(la) * h2g_ncart(lb);
    double acc[H2G_NCUM(H2G_MAX_L)];
    double work[2 * H2G_NCUM(H2G_MAX_L) * 16];
    double res[H2G_NCUM(H2G_MAX_L) * H2G_NCUM(H2G_MAX_L)];
    const double Av[3] = {A->x, A->y, A->z}, Bv[3] = {B->x, B->y, B->z};
    double ab2 = 0.0;
    for (int d = 0; d < 3; d++) ab2 += (Av[d] - Bv[d]) * (Av[d] - Bv[d]);
    /* primitive-pair data, shared by all points: p, K, P[3] */
    const int npp = A->nprim * B->nprim;
    double *pp = (double *)malloc(sizeof(double) * 5 * (size_t)(npp > 0 ? npp : 1));
    for (int i = 0; i < A->nprim; i++)
        for (int j = 0; j < B->nprim; j++) {
            const double a = A->alpha[i], b = B->alpha[j], p = a + b;
            double *q = pp + 5 * (i * B->nprim + j);
            q[0] = p;
            q[1] = A->coef[i] * B->coef[j] * exp(-a * b / p * ab2);
            for (int d = 0; d < 3; d++) q[2 + d] = (a * Av[d] + b * Bv[d]) / p;
        }
    const double ABv[3] = {Av[0] - Bv[0], Av[1] - Bv[1], Av[2] - Bv[2]};
    /* H2G_LANES points at a time (lanes past n_pt repeat the last point and
     * are discarded) */
    vlane Vl[H2G_NCUM(H2G_MAX_L) * (H2G_MAX_L + 1)], accl[H2G_NCUM(H2G_MAX_L)];
    for (int pt0 = 0; pt0 < n_pt; pt0 += H2G_LANES) {
        vlane C[3];
        for (int l = 0; l < H2G_LANES; l++) {
            const int pt = (pt0 + l < n_pt) ? pt0 + l : n_pt - 1;
            C[0][l] = cx[pt];
            C[1][l] = cy[pt];
            C[2][l] = cz[pt];
        }
        for (int e = 0; e < ne; e++) accl[e] = (vlane){0.0, 0.0, 0.0, 0.0};
        for (int k = 0; k < npp; k++) {
            const double *q = pp + 5 * k;
            const double p = q[0], K = q[1], *P = q + 2;
            double PA[3];
            vlane PC[3], PC2 = {0.0, 0.0, 0.0, 0.0};
            for (int d = 0; d < 3; d++) {
                PA[d] = P[d] - Av[d];
                PC[d] = P[d] - C[d];
                PC2 += PC[d] * PC[d];
            }
            double F[H2G_LANES][H2G_MAX_L + 1];
            for (int l = 0; l < H2G_LANES; l++) h2g_boys(L, p * PC2[l], F[l]);
            const double pref = -charge * 2.0 * M_PI / p * K;
            for (int m = 0; m <= L; m++)
                for (int l = 0; l < H2G_LANES; l++) Vl[m][l] = pref * F[l][m];
            const double i2p = 0.5 / p;
            /* [e+1_i]^(m) = PA_i [e]^(m) - PC_i [e]^(m+1) + e_i/(2p) ([e-1_i]^(m) - [e-1_i]^(m+1)) */
            for (int c = 1; c < ne; c++) {
                const int Lc = g_lxyz[c][0] + g_lxyz[c][1] + g_lxyz[c][2];
                const int d = g_dir[c], e = g_prev[c], e2 = g_prev2[c];
                const double ei = (double)(g_lxyz[c][d] - 1);
                for (int m = 0; m <= L - Lc; m++) {
                    vlane v = PA[d] * Vl[e * nm + m] - PC[d] * Vl[e * nm + m + 1];
                    if (e2 >= 0) v += ei * i2p * (Vl[e2 * nm + m] - Vl[e2 * nm + m + 1]);
                    Vl[c * nm + m] = v;
                }
            }
            for (int e = g_cum[la]; e < ne; e++) accl[e] += Vl[e * nm];
        }
        for (int l = 0; l < H2G_LANES && pt0 + l < n_pt; l++) {
            for (int e = 0; e < ne; e++) acc[e] = accl[e][l];
            hrr(la, lb, ABv, acc, 1, res, work);
            for (int r = 0; r < nab; r++) out[(size_t)r * ldo + pt0 + l] = res[r];
        }
    }
    free(pp);
}

void h2g_potential(const h2g_shell *A, const h2g_shell *B,
                   double cx, double cy, double cz, double charge, double *out)
{
    h2g_potential_points(A, B, 1, &cx, &cy, &cz, charge, out, 1);
}
