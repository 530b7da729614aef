/*
 * Test-infrastructure shim: the SIMINT API subset the reference uses,
 * implemented on the project's integral engine. Compiled only into the
 * oracle library built from the reference sources (oracle/build_ref.py).
 */
#include <stdlib.h>
#include <string.h>

#include "simint/simint.h"
#include "h2g_ints.h"

void simint_init(void) { h2g_ints_init(); }
void simint_finalize(void) {}

void *simint_shim_alloc(size_t sz)
{
    void *p = NULL;
    if (posix_memalign(&p, 64, sz > 0 ? sz : 64) != 0) return NULL;
    return p;
}
void simint_shim_free(void *p) { free(p); }

void simint_initialize_shell(struct simint_shell *G) { memset(G, 0, sizeof(*G)); }
void simint_initialize_shells(int n, struct simint_shell *G)
{
    for (int i = 0; i < n; i++) simint_initialize_shell(&G[i]);
}

void simint_allocate_shell(int nprim, struct simint_shell *G)
{
    free(G->alpha);
    free(G->coef);
    G->alpha = (double *)calloc((size_t)(nprim > 0 ? nprim : 1), sizeof(double));
    G->coef = (double *)calloc((size_t)(nprim > 0 ? nprim : 1), sizeof(double));
    G->memsize = sizeof(double) * 2 * (size_t)nprim;
}

void simint_free_shell(struct simint_shell *G)
{
    free(G->alpha);
    free(G->coef);
    G->alpha = G->coef = NULL;
    G->memsize = 0;
}

void simint_copy_shell(const struct simint_shell *src, struct simint_shell *dest)
{
    dest->am = src->am;
    dest->nprim = src->nprim;
    dest->x = src->x; dest->y = src->y; dest->z = src->z;
    memcpy(dest->alpha, src->alpha, sizeof(double) * (size_t)src->nprim);
    memcpy(dest->coef, src->coef, sizeof(double) * (size_t)src->nprim);
}

void simint_normalize_shells(int n, struct simint_shell *G)
{
    for (int i = 0; i < n; i++) h2g_normalize_shell(G[i].am, G[i].nprim, G[i].alpha, G[i].coef);
}

static void to_h2g(const struct simint_shell *s, h2g_shell *t)
{
    t->am = s->am; t->nprim = s->nprim;
    t->x = s->x; t->y = s->y; t->z = s->z;
    t->alpha = s->alpha; t->coef = s->coef;
}

void simint_initialize_multi_shellpair(struct simint_multi_shellpair *P) { memset(P, 0, sizeof(*P)); }

void simint_free_multi_shellpair(struct simint_multi_shellpair *P)
{
    if (P->owns)
        for (int i = 0; i < P->nshell12; i++) {
            h2g_pair_free((h2g_pair *)P->pairs[i]);
            free(P->pairs[i]);
        }
    free(P->pairs);
    memset(P, 0, sizeof(*P));
}

void simint_create_multi_shellpair(int na, const struct simint_shell *A,
                                   int nb, const struct simint_shell *B,
                                   struct simint_multi_shellpair *P, int screen_method)
{
    (void)screen_method;
    simint_free_multi_shellpair(P);
    P->pairs = (void **)malloc(sizeof(void *) * (size_t)(na * nb));
    P->capacity = na * nb;
    P->owns = 1;
    P->am1 = A[0].am;
    P->am2 = B[0].am;
    for (int i = 0; i < na; i++)
        for (int j = 0; j < nb; j++) {
            h2g_shell a, b;
            to_h2g(&A[i], &a);
            to_h2g(&B[j], &b);
            h2g_pair *pr = (h2g_pair *)malloc(sizeof(h2g_pair));
            h2g_pair_init(pr, &a, &b);
            P->pairs[P->nshell12++] = pr;
            P->nprim += pr->nprim;
        }
}

void simint_cat_shellpairs(int nmpair, const struct simint_multi_shellpair **P,
                           struct simint_multi_shellpair *out, int screen_method)
{
    (void)screen_method;
    int total = 0;
    for (int i = 0; i < nmpair; i++) total += P[i]->nshell12;
    if (out->owns) simint_free_multi_shellpair(out);
    if (out->capacity < total) {
        free(out->pairs);
        out->pairs = (void **)malloc(sizeof(void *) * (size_t)total);
        out->capacity = total;
    }
    out->owns = 0;
    out->nshell12 = 0;
    out->nprim = 0;
    if (nmpair > 0) { out->am1 = P[0]->am1; out->am2 = P[0]->am2; }
    for (int i = 0; i < nmpair; i++)
        for (int k = 0; k < P[i]->nshell12; k++) {
            out->pairs[out->nshell12++] = P[i]->pairs[k];
            out->nprim += ((h2g_pair *)P[i]->pairs[k])->nprim;
        }
}

size_t simint_ostei_workmem(int derorder, int maxam)
{
    (void)derorder; (void)maxam;
    return 64;   /* the engine keeps its scratch in thread-local storage */
}

int simint_compute_eri(const struct simint_multi_shellpair *P,
                       const struct simint_multi_shellpair *Q,
                       double screen_tol, double *work, double *integrals)
{
    (void)screen_tol; (void)work;
    int n = 0;
    int sz = h2g_ncart(P->am1) * h2g_ncart(P->am2) * h2g_ncart(Q->am1) * h2g_ncart(Q->am2);
    for (int i = 0; i < P->nshell12; i++)
        for (int j = 0; j < Q->nshell12; j++) {
            h2g_eri_quartet((const h2g_pair *)P->pairs[i], (const h2g_pair *)Q->pairs[j],
                            integrals + (size_t)n * sz);
            n++;
        }
    return n;
}

int simint_compute_potential(int ncenter, const double *Z,
                             const double *x, const double *y, const double *z,
                             const struct simint_shell *sh1, const struct simint_shell *sh2,
                             double *integrals)
{
    h2g_shell a, b;
    to_h2g(sh1, &a);
    to_h2g(sh2, &b);
    int sz = h2g_ncart(a.am) * h2g_ncart(b.am);
    double tmp[15 * 15];
    memset(integrals, 0, sizeof(double) * (size_t)sz);
    for (int c = 0; c < ncenter; c++) {
        h2g_potential(&a, &b, x[c], y[c], z[c], Z[c], tmp);
        for (int k = 0; k < sz; k++) integrals[k] += tmp[k];
    }
    return 1;
}
