/*
 * Test-infrastructure driver compiled into the oracle library next to the
 * unmodified reference sources. It runs the reference's own set-up sequence
 * (as in H2P-ERI tests/test_J_input_mat.c:17-31) and exposes a few struct
 * fields to Python without a struct mirror.
 */
#include <stdlib.h>
#include <string.h>
#include "H2ERI.h"

H2ERI_p oref_build(const char *mol, double scr_tol, double ext_tol, double qr_tol, int bd_jit)
{
    H2ERI_p h2eri;
    simint_init();
    H2ERI_init(&h2eri, scr_tol, ext_tol, qr_tol);
    CMS_read_mol_file(mol, &h2eri->natom, &h2eri->nshell, &h2eri->shells);
    H2ERI_process_shells(h2eri);
    H2ERI_partition(h2eri);
    H2ERI_build_H2(h2eri, bd_jit);
    return h2eri;
}

int oref_num_bf(H2ERI_p h) { return h->num_bf; }
int oref_krnl_mat_size(H2ERI_p h) { return h->krnl_mat_size; }
int oref_n_thread(H2ERI_p h) { return h->n_thread; }
size_t oref_struct_size(void) { return sizeof(struct H2ERI); }
void oref_reset_timers(H2ERI_p h) { h->n_matvec = 0; memset(h->timers + 4, 0, sizeof(double) * 5); }
