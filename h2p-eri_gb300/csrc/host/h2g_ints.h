/*
 * Gaussian integral engine used by the per-geometry H2 construction.
 *
 * The reference delegates electron-repulsion integrals (ERI) and point-charge
 * potential integrals to the external SIMINT library
 * (H2P-ERI src/CMS.c:163-229, 268-482). SIMINT is an external dependency
 * that this library does not take, so this file provides an independent
 * implementation of the same integrals:
 *
 *   - Cartesian Gaussian shells, all Cartesian components of a shell share one
 *     contracted coefficient set (SIMINT convention, see h2g_normalize_shell);
 *   - component order inside a shell of angular momentum L is lexicographic in
 *     decreasing x power, then decreasing y power (xx, xy, xz, yy, yz, zz);
 *   - a shell quartet (AB|CD) is written row-major as [a][b][c][d];
 *   - a potential integral <A|1/|r-C||B> is written row-major as [a][b].
 *
 * Method: Obara-Saika vertical recurrence on primitive quartets, contraction,
 * then the Head-Gordon-Pople horizontal recurrence on contracted quantities
 * (M. Head-Gordon, J. A. Pople, J. Chem. Phys. 89, 5777 (1988); S. Obara,
 * A. Saika, J. Chem. Phys. 84, 3963 (1986)). The Boys function uses a
 * pretabulated grid with a 7-term Taylor expansion below T = 40 and the
 * asymptotic form with upward recursion above it (T. Helgaker, P. Jorgensen,
 * J. Olsen, Molecular Electronic-Structure Theory, Wiley 2000, sec. 9.8).
 *
 * This is host code only; it is not part of the GPU hot path.
 */
#ifndef H2G_INTS_H
#define H2G_INTS_H

#ifdef __cplusplus
extern "C" {
#endif

#define H2G_MAX_AM 4   /* per shell; cc-pVDZ needs 2 */

/* Number of Cartesian components of angular momentum am. */
static inline int h2g_ncart(int am) { return (am + 1) * (am + 2) / 2; }

/* One contracted Cartesian shell. coef[] already carries normalisation. */
typedef struct h2g_shell_s {
    int am, nprim;
    double x, y, z;
    const double *alpha;
    const double *coef;
} h2g_shell;

/* Precomputed primitive-pair data for a shell pair (A, B). */
typedef struct h2g_pair_s {
    int am1, am2;        /* angular momenta of A and B */
    int nprim;           /* number of kept primitive pairs */
    double A[3], B[3];   /* shell centres */
    double *P;           /* [nprim][3] Gaussian product centres */
    double *p;           /* [nprim] exponent sums a + b */
    double *K;           /* [nprim] c_a c_b exp(-a b / p |AB|^2) */
    double *ip;          /* [nprim] 1 / p */
} h2g_pair;

/* Build primitive-pair data; primitive pairs whose prefactor magnitude falls
 * below 1e-30 are dropped (contribution far below double rounding). */
void h2g_pair_init(h2g_pair *pr, const h2g_shell *A, const h2g_shell *B);
void h2g_pair_free(h2g_pair *pr);

/* Contracted ERI (AB|CD) for bra pair (A,B) and ket pair (C,D).
 * out: ncart(A)*ncart(B)*ncart(C)*ncart(D) doubles, row-major [a][b][c][d]. */
void h2g_eri_quartet(const h2g_pair *bra, const h2g_pair *ket, double *out);

/* Potential integral of a unit positive point charge at (cx,cy,cz):
 * out[a][b] = -charge * < A_a | 1/|r - C| | B_b >  (attraction sign). */
void h2g_potential(const h2g_shell *A, const h2g_shell *B,
                   double cx, double cy, double cz, double charge, double *out);

/* The same for n_pt charges at (cx[k], cy[k], cz[k]), the primitive-pair
 * data formed once: out[ab * ldo + k] is component ab (row-major [a][b]) at
 * point k. */
void h2g_potential_points(const h2g_shell *A, const h2g_shell *B, int n_pt, const double *cx,
                          const double *cy, const double *cz, double charge, double *out, int ldo);

/* Boys function F_m(T) for m = 0..mmax (mmax <= 4*H2G_MAX_AM). */
void h2g_boys(int mmax, double T, double *F);

/* Normalise coefficients in place (SIMINT convention): after the call the
 * contracted function built from the x^L component has unit norm, and every
 * coef[k] includes the primitive factor alpha[k]^((L+1.5)/2).
 * Input coef are the raw contraction coefficients of the basis file. */
void h2g_normalize_shell(int am, int nprim, const double *alpha, double *coef);

/* Initialise the Boys-function table (thread-safe, idempotent). */
void h2g_ints_init(void);

/* Copies of the engine's tables, for a device implementation of the same
 * recurrences: Cartesian components over total L <= 2 * H2G_MAX_AM
 * (lxyz[c][3], cum[L + 2] first index of each L, dir / prev / prev2 of the
 * recurrence, minus[c][3] / plus[c][3] neighbours) and the Boys-function grid
 * (boys[k][m], k over 0, 0.05, ..., 40). dims gets {max L, components,
 * grid points, orders per grid point}; a NULL table is skipped. */
int h2g_ints_tables(int *lxyz, int *cum, int *dir, int *prev, int *prev2, int *minus, int *plus, double *boys,
                    int *dims);

#ifdef __cplusplus
}
#endif

#endif
