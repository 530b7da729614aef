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
/* 1 when the set-up may use the GPU: a CUDA device is present and the
 * environment does not set H2G_SETUP_GPU=0. */
int gpu_eri_usable();

}  // namespace h2g

#endif
