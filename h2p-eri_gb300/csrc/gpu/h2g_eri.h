/*
 * GPU evaluation of electron-repulsion integral blocks for the host set-up
 * (h2g_eri.cu). No CUDA types: the host set-up code includes this header.
 */
#ifndef H2G_ERI_H
#define H2G_ERI_H

#include <vector>

#include "h2g_ints.h"

namespace h2g {

struct EriSet;   /* one structure's shell pairs on the device */

/* One block of shell quartets (NM|QP): rows are the bf pairs of the bra
 * shell pairs in order, columns those of the ket pairs (the layout of the
 * host eri_pairs_to_mat). With `sym` (bra == ket, a diagonal block) only
 * quartets with bra position <= ket position are evaluated and mirrored.
 * The block is written to out (row-major, leading dimension ld); nrow and
 * ncol are set by the call. */
struct EriReq {
    std::vector<int> bra, ket;
    bool sym = false;
    double *out = nullptr;
    int ld = 0;
    int nrow = 0, ncol = 0;
};

/* Upload the primitive-pair data of n_sp shell pairs (index = shell-pair
 * index of the structure). Returns 0, or 3 when a shell is above d (the
 * host engine then stays in use), or another error code. */
int gpu_eri_create(int n_sp, const h2g_pair *const *pairs, EriSet **out);
/* Evaluate the blocks of reqs on the device and copy them into their host
 * matrices. Returns 0 or an error code (message in H2ERI_gpu_last_error). */
int gpu_eri_blocks(EriSet *s, std::vector<EriReq> &reqs);
void gpu_eri_free(EriSet *s);

/* The sketched integral matrix of one node of the nested-basis (U) set-up:
 * rows = the bf pairs of the bra shell pairs in order; columns [0, nrow) =
 * the potentials of npt unit point charges (px/py/pz) times a sparse sign
 * sketch (column j = sum over l < s1_nnz of s1_val[j s1_nnz + l] times the
 * potential column s1_col[j s1_nnz + l]); columns [nrow, 2 nrow) = the ERIs
 * with the ket shell pairs (columns = their bf pairs in order) times the
 * second sketch in the same form. All pointers are host memory owned by the
 * caller; out is nrow x 2 nrow with leading dimension ld. nrow and ncol_ff
 * (ket bf pairs) are set by the call. */
struct UReq {
    const int *bra = nullptr, *ket = nullptr;
    int nbra = 0, nket = 0;
    const double *px = nullptr, *py = nullptr, *pz = nullptr;
    int npt = 0;
    const int *s1_col = nullptr, *s2_col = nullptr;
    const double *s1_val = nullptr, *s2_val = nullptr;
    int s1_nnz = 0, s2_nnz = 0;
    double *out = nullptr;
    int ld = 0;
    int nrow = 0, ncol_ff = 0;
};
/* Evaluate the requests on the device (potentials, ERIs and both sketches)
 * and copy each sketched matrix into its host matrix. Returns 0 or an error
 * code (message in H2ERI_gpu_last_error). */
int gpu_u_blocks(EriSet *s, std::vector<UReq> &reqs);
/* 1 when the set-up may use the GPU: a CUDA device is present and the
 * environment does not set H2G_SETUP_GPU=0. */
int gpu_eri_usable();

}  // namespace h2g

#endif
