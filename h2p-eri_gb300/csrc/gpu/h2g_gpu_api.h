/* Internal cross-file interface of the GPU part (not exported). */
#ifndef H2G_GPU_API_H
#define H2G_GPU_API_H

#include <string>
#include <cuda_runtime.h>
#include "h2eri_types.h"
#include "h2g_device.cuh"
#include <nvtx3/nvToolsExt.h>

/* A named range for profilers (NVTX; header-only, inert unless a tool such
 * as Nsight Systems is attached) around each hot-path entry point. */
struct H2gRange {
    explicit H2gRange(const char *name) { nvtxRangePushA(name); }
    ~H2gRange() { nvtxRangePop(); }
    H2gRange(const H2gRange &) = delete;
    H2gRange &operator=(const H2gRange &) = delete;
};

namespace h2g {

void set_error(const std::string &msg);
/* device representation of h, uploaded on first use */
int get_rep(H2ERI_p h, DevRep **out);
/* y = A x on device vectors, enqueued on s */
int enqueue_matvec(DevRep *d, int nvec, const double *x, double *y, cudaStream_t s, bool timed);
int enqueue_coulomb(DevRep *d, int n_den, const double *den, double *J, cudaStream_t s, bool timed,
                    bool den_in_host = false);   /* den_in_host: page-locked host memory, read in place */
/* exchange state attached to a representation */
void free_exchange_state(DevRep *d);
int ensure_work(DevRep *d, int nvec);
/* single-density tile plan rebuilt with other tile rows (autotuning) */
int replan_tiles(DevRep *d, int rows);
/* launch choices from the tuning cache (H2G_TUNE_FILE), at upload */
void tune_apply_cached(DevRep *d);
int enqueue_uncontract(DevRep *d, int n_den, const double *den, cudaStream_t s);
int enqueue_contract(DevRep *d, int n_den, double *J, cudaStream_t s);
/* batched J over several structures in shared launches (h2g_batch.cu) */
int batch_merged_kind(int n, DevRep *const *reps, const int *n_den);
int batch_coulomb_merged(int kind, int n, DevRep *const *reps, const int *n_den, const double *const *d_dens,
                         double *const *d_Js, cudaStream_t s);
void batch_forget(const DevRep *d);
/* multi-density tensor-core kernel (h2g_mma.cu) */
int mma_init(DevRep *d);
int mma_make_slices(DevRep *d);
void launch_range_mma(const DevRep *d, const Range &r, const VecArgs &va, int nvec, cudaStream_t s);
/* a merged range of a batch plan on the mixed single-density kernel */
void launch_batch_mx(const Tile *tiles, int count, bool pair, const void *maps, const BatchMol *mols, int nvec,
                     int tiles_per_cta, unsigned *err, cudaStream_t s);
/* a range of a batch plan: tiles, their scales and the structures' table */
void launch_batch_mma(const TileM *tiles, const int8_t *scales, const BatchMol *mols, int count, int levels, int n_sm,
                      unsigned *err, cudaStream_t s);
/* precision switch (mixed far-field arenas) */
int set_precision_mode(DevRep *d, H2ERI_p h, int mode);

}  // namespace h2g

#endif
