/*
 * Data types shared with callers of the H2P-ERI C API.
 *
 * Callers write and read fields of struct H2ERI directly (H2P-ERI
 * tests/test_J_input_mat.c:22,34,47-48 write natom/nshell/shells and read
 * num_bf, n_matvec, timers), so the field order and types below follow the
 * reference layout exactly (H2P-ERI src/H2ERI_typedef.h:14-131,
 * src/H2ERI_aux_structs.h:12-23,41-46,150-157,284-293, src/CMS.h:7-45).
 * Memory inside the struct is owned by the library and released by
 * H2ERI_destroy().
 *
 * The GPU state of a struct (device copies of U/B/D and tree arrays) is not
 * stored in the struct; the library keeps it in a side table keyed by the
 * H2ERI_p pointer (see h2eri_gb300.h: H2ERI_gpu_release).
 */
#ifndef H2ERI_TYPES_H
#define H2ERI_TYPES_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- integral-library shell types (layout of SIMINT's shell struct) ---- */
struct simint_shell {
    int am;            /* angular momentum                         */
    int nprim;         /* number of primitives                     */
    double x, y, z;    /* centre, Bohr                             */
    double *alpha;     /* [nprim] exponents                        */
    double *coef;      /* [nprim] normalised contraction coeffs    */
    size_t memsize;
    void *ptr;
};
typedef struct simint_shell shell_t;
typedef struct simint_shell *shell_p;

/* Shell pair: opaque to the hot path; the set-up code stores primitive-pair
 * data here. Only am1/am2 are read by generic code. */
struct simint_multi_shellpair {
    int am1, am2;
    int nprim;
    int nshell12;
    int owns;
    int capacity;
    void **pairs;
};
typedef struct simint_multi_shellpair multi_sp_t;
typedef struct simint_multi_shellpair *multi_sp_p;

/* Per-thread integral buffers (opaque here). */
typedef struct simint_buff *simint_buff_p;
typedef struct eri_batch_buff *eri_batch_buff_p;

#define NCART(am) ((am >= 0) ? ((((am) + 2) * ((am) + 1)) >> 1) : 0)

/* ---- auxiliary containers ---- */
struct H2E_int_vec {
    int capacity;
    int length;
    int *data;
};
typedef struct H2E_int_vec *H2E_int_vec_p;

/* Dense row-major matrix. ld > 0: dense nrow x ncol with leading dimension ld.
 * ld = -r < 0 (B and D blocks only): low-rank form, data holds U (nrow x r,
 * row-major) followed by V^T (ncol x r, row-major) so the block is U * V. */
struct H2E_dense_mat {
    int nrow;
    int ncol;
    int ld;
    int size;
    double *data;
};
typedef struct H2E_dense_mat *H2E_dense_mat_p;

struct H2E_thread_buf {
    H2E_int_vec_p idx0;
    H2E_int_vec_p idx1;
    H2E_dense_mat_p mat0;
    H2E_dense_mat_p mat1;
    H2E_dense_mat_p mat2;
    double *y;          /* krnl_mat_size partial matvec output */
    double timer;
};
typedef struct H2E_thread_buf *H2E_thread_buf_p;

/* ---- the H2 representation of the ERI tensor ---- */
struct H2ERI {
    int    natom;
    int    nshell;
    int    max_am;
    int    max_shell_nbf;
    int    num_bf;
    int    num_sp;                  /* screened shell pairs (SSP)                    */
    int    num_sp_bfp;              /* SSP basis-function pairs == krnl_mat_size     */
    int    pp_npts_layer;
    int    pp_nlayer_ext;
    int    *shell_bf_sidx;          /* [nshell+1]                                    */
    int    *sp_nbfp;                /* [num_sp]                                      */
    int    *sp_bfp_sidx;            /* [num_sp+1]                                    */
    int    *sp_shell_idx;           /* [2*num_sp]: shell M (i) and shell N (num_sp+i)*/
    int    *index_seq;
    int    *node_adm_pairs;
    int    *node_adm_pairs_sidx;
    int    *node_inadm_pairs;
    int    *node_inadm_pairs_sidx;
    int    *plist;
    int    *plist_idx;
    int    *plist_sidx;
    int    *dlist;
    int    *dlist_sidx;
    void   **thread_Kmat_workbuf;
    double scr_tol;
    double ext_tol;
    double *sp_center;
    double *sp_extent;
    double *box_extent;
    double *unc_denmat_x;
    double *H2_matvec_y;
    shell_t          *shells;
    shell_t          *sp_shells;
    multi_sp_t       *sp;
    H2E_int_vec_p    *J_pair;
    H2E_int_vec_p    *J_row;
    H2E_int_vec_p    *ovlp_ff_idx;
    simint_buff_p    *simint_buffs;
    eri_batch_buff_p *eri_batch_buffs;
    H2E_dense_mat_p  *c_B_blks;     /* [n_B] coupling blocks (dense or low-rank)     */
    H2E_dense_mat_p  *c_D_blks;     /* [n_D] near-field blocks (dense or low-rank)   */
    H2E_thread_buf_p *thread_buffs;

    int    n_thread;
    int    pt_dim;
    int    xpt_dim;
    int    krnl_dim;
    int    QR_stop_type;
    int    QR_stop_rank;
    int    n_point;
    int    krnl_mat_size;
    int    max_leaf_points;
    int    n_node;
    int    root_idx;
    int    n_leaf_node;
    int    max_child;
    int    max_neighbor;
    int    max_level;
    int    min_adm_level;
    int    n_r_inadm_pair;
    int    n_r_adm_pair;
    int    n_UJ;
    int    n_B;
    int    n_D;
    int    BD_JIT;
    int    print_timers;
    int    print_dbginfo;
    int    *parent;
    int    *children;               /* [n_node * max_child]                          */
    int    *pt_cluster;             /* [2*n_node] inclusive SSP ranges               */
    int    *mat_cluster;            /* [2*n_node] inclusive vector ranges            */
    int    *n_child;
    int    *node_level;
    int    *node_height;
    int    *level_n_node;
    int    *level_nodes;            /* [(max_level+1) * n_leaf_node]                 */
    int    *height_n_node;
    int    *height_nodes;           /* height 0 row == leaf nodes                    */
    int    *r_inadm_pairs;
    int    *r_adm_pairs;
    int    *node_inadm_lists;
    int    *node_n_r_inadm;
    int    *node_n_r_adm;
    int    *coord_idx;
    int    *B_p2i_rowptr;
    int    *B_p2i_colidx;
    int    *B_p2i_val;
    int    *D_p2i_rowptr;
    int    *D_p2i_colidx;
    int    *D_p2i_val;
    int    *B_nrow;
    int    *B_ncol;
    int    *D_nrow;
    int    *D_ncol;
    size_t *B_ptr;
    size_t *D_ptr;
    double max_leaf_size;
    double QR_stop_tol;
    double *coord;
    double *coord0;
    double *enbox;
    double *root_enbox;
    double *B_data;
    double *D_data;
    H2E_int_vec_p   B_blk;
    H2E_int_vec_p   D_blk0;
    H2E_int_vec_p   D_blk1;
    H2E_dense_mat_p *U;             /* [n_node] nested bases, row-major nrow x ncol  */
    H2E_dense_mat_p *y0;
    H2E_dense_mat_p *y1;
    int    n_matvec;
    size_t mat_size[11];
    double timers[11];
};
typedef struct H2ERI *H2ERI_p;

/* mat_size[] slots (element counts) */
enum {
    U_SIZE_IDX = 0, B_SIZE_IDX, D_SIZE_IDX,
    MV_FWD_SIZE_IDX, MV_MID_SIZE_IDX, MV_BWD_SIZE_IDX, MV_DEN_SIZE_IDX, MV_VOP_SIZE_IDX
};
/* timers[] slots (seconds) */
enum {
    PT_TIMER_IDX = 0, U_BUILD_TIMER_IDX, B_BUILD_TIMER_IDX, D_BUILD_TIMER_IDX,
    MV_FWD_TIMER_IDX, MV_MID_TIMER_IDX, MV_BWD_TIMER_IDX, MV_DEN_TIMER_IDX, MV_VOP_TIMER_IDX
};

#ifdef __cplusplus
}
#endif

#endif
