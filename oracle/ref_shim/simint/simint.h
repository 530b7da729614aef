/*
 * Test-infrastructure shim: declares exactly the subset of the SIMINT API
 * (simint-generator commit a497ec7, "simint-2022Apr14", not vendored) that
 * the reference H2P-ERI sources call, so they compile unchanged into the
 * oracle library. Implemented in ../simint_shim.c on top of the project's
 * own integral engine (h2p-eri_gb300/csrc/host/h2g_ints.c).
 *
 * Call sites in the reference: src/CMS.c:118,163-229,268-360,455-482,
 * src/H2ERI_partition.c:67-96, src/H2ERI_shell_operations.c:48-80.
 * Only this header's names and argument meanings follow SIMINT; the struct
 * layouts carry just the fields the reference reads (am, nprim, x, y, z,
 * alpha, coef; am1, am2, nprim).
 */
#ifndef ORACLE_SIMINT_SHIM_H
#define ORACLE_SIMINT_SHIM_H

#include <stddef.h>
/* The real SIMINT headers pull these in; the reference relies on them. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SIMINT_SCREEN_NONE 0

struct simint_shell {
    int am;
    int nprim;
    double x, y, z;
    double *alpha;
    double *coef;
    size_t memsize;
    void *ptr;
};

struct simint_multi_shellpair {
    int am1, am2;
    int nprim;          /* total primitive pairs (informational) */
    int nshell12;       /* number of component shell pairs        */
    int owns;           /* 1 if pairs[] are owned by this object   */
    int capacity;
    void **pairs;       /* h2g_pair* per component shell pair     */
};

void simint_init(void);
void simint_finalize(void);

void simint_initialize_shell(struct simint_shell *G);
void simint_initialize_shells(int n, struct simint_shell *G);
void simint_allocate_shell(int nprim, struct simint_shell *G);
void simint_free_shell(struct simint_shell *G);
void simint_copy_shell(const struct simint_shell *src, struct simint_shell *dest);
void simint_normalize_shells(int n, struct simint_shell *G);

void simint_initialize_multi_shellpair(struct simint_multi_shellpair *P);
void simint_free_multi_shellpair(struct simint_multi_shellpair *P);
void simint_create_multi_shellpair(int na, const struct simint_shell *A,
                                   int nb, const struct simint_shell *B,
                                   struct simint_multi_shellpair *P, int screen_method);
void simint_cat_shellpairs(int nmpair, const struct simint_multi_shellpair **P,
                           struct simint_multi_shellpair *out, int screen_method);

size_t simint_ostei_workmem(int derorder, int maxam);
int simint_compute_eri(const struct simint_multi_shellpair *P,
                       const struct simint_multi_shellpair *Q,
                       double screen_tol, double *work, double *integrals);
int simint_compute_potential(int ncenter, const double *Z,
                             const double *x, const double *y, const double *z,
                             const struct simint_shell *sh1, const struct simint_shell *sh2,
                             double *integrals);

void *simint_shim_alloc(size_t sz);
void simint_shim_free(void *p);
#define SIMINT_ALLOC(sz) simint_shim_alloc(sz)
#define SIMINT_FREE(p)   simint_shim_free(p)

#ifdef __cplusplus
}
#endif

#endif
