/*
 * Internal host-side helpers shared by the set-up (H2 construction) files.
 * Not part of the public C API.
 */
#ifndef H2G_HOST_H
#define H2G_HOST_H

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "h2eri_types.h"
#include "h2g_ints.h"

#define H2G_ALPHA_H2   0.999999   /* admissibility coefficient (H2P-ERI src/H2ERI_config.h:56) */
#define H2G_ALPHA_SUP  1.0        /* super-cell coefficient (H2P-ERI src/H2ERI_typedef.h:160)  */
#define H2G_BD_NTASK   10         /* tasks per thread in B/D partition (src/H2ERI_config.h:59) */

#define H2G_FATAL(...)                                                       \
    do {                                                                     \
        std::fprintf(stderr, "[h2eri_gb300 FATAL] %s:%d: ", __FILE__, __LINE__); \
        std::fprintf(stderr, __VA_ARGS__);                                   \
        std::fflush(stderr);                                                 \
        std::abort();                                                        \
    } while (0)

#define H2G_CHECK(cond, ...) do { if (!(cond)) H2G_FATAL(__VA_ARGS__); } while (0)

namespace h2g {

double wtime();
void *amalloc(size_t bytes);            /* 64-byte aligned, freed with free() */

/* H2E_int_vec / H2E_dense_mat helpers with the reference semantics
 * (H2P-ERI src/H2ERI_aux_structs.c). */
H2E_int_vec_p ivec_new(int capacity);
void ivec_free(H2E_int_vec_p *v);
void ivec_reserve(H2E_int_vec_p v, int capacity);
void ivec_push(H2E_int_vec_p v, int x);
H2E_dense_mat_p dmat_new(int nrow, int ncol);
void dmat_free(H2E_dense_mat_p *m);
void dmat_resize(H2E_dense_mat_p m, int nrow, int ncol);
H2E_thread_buf_p tbuf_new(int krnl_mat_size);
void tbuf_free(H2E_thread_buf_p *tb);
void tbuf_reset(H2E_thread_buf_p tb);

/* Integral helpers on SSP shell pairs (row order (N,M): N-major, M-minor,
 * H2P-ERI src/CMS.h:138-158). */
h2g_pair *sp_pair(H2ERI_p h2eri, int sp_idx);
void eri_pairs_to_mat(H2ERI_p h2eri, int n_bra, const int *bra, int n_ket, const int *ket,
                      double *mat, int ldm);
void nai_pairs_to_mat(H2ERI_p h2eri, int n_bra, const int *bra, int n_pt,
                      const double *x, const double *y, const double *z, double *mat, int ldm);

/* Work partition into blocks of about equal total size (src/H2ERI_utils.c:168-195). */
void partition_workload(int n_work, const size_t *work_sizes, size_t total, int n_block,
                        H2E_int_vec_p displs);

/* Interpolative decomposition over rows (src/H2E_ID_compress.c:491-576). A is
 * row-major nrow x ncol and is destroyed. On return J holds the sorted skeleton
 * row indices and, if U_out != NULL, *U_out is the nrow x r projection. */
void id_compress(H2E_dense_mat_p A, double rel_tol, H2E_dense_mat_p *U_out, H2E_int_vec_p J);

void build_h2(H2ERI_p h2eri);

}  // namespace h2g

/* id_compress on a copy of a row-major nrow x ncol matrix, for tests through
 * the shared library: returns the rank r, J[0..r) the sorted skeleton rows,
 * U (nrow x r, row-major, room for nrow * min(nrow, ncol) values). */
extern "C" int h2g_id_rows(int nrow, int ncol, const double *A, double rel_tol, int *J, double *U);

#endif
