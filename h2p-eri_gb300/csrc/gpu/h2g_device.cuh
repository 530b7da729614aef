/*
 * Internal GPU data structures of the H2 apply (device representation of one
 * struct H2ERI). Host-only declarations plus the tile descriptor shared with
 * the kernels.
 */
#ifndef H2G_DEVICE_CUH
#define H2G_DEVICE_CUH

#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "h2eri_types.h"

namespace h2g {

/* Vector spaces a tile reads from / accumulates into. */
enum VecKind : uint8_t {
    VK_NONE = 0,
    VK_X = 1,    /* matvec input x        [nvec][krnl_mat_size]  */
    VK_Y = 2,    /* matvec output y       [nvec][krnl_mat_size]  */
    VK_Y0 = 3,   /* upward coefficients   [nvec][rank_total]     */
    VK_Y1 = 4,   /* downward coefficients [nvec][rank_total]     */
    VK_T = 5,    /* low-rank scratch      [nvec][lr_total]       */
    VK_COUNT = 6
};

/* One tile of one stored matrix (a U basis, a B or D block, or a factor of a
 * low-rank block): rows [r0, r0+nr), columns [c0, c0+nc) of a row-major
 * matrix with leading dimension ld. Two optional products:
 *   N: out0[r] += sum_c A[r][c] * in0[c]
 *   T: out1[c] += sum_r A[r][c] * in1[r]
 * Offsets are element offsets (already shifted by r0 / c0) into the vector
 * space named by the kind byte. */
struct Tile {
    uint64_t a;            /* element offset of A[r0][c0] in the FP64 arena              */
    uint64_t a2;           /* mixed formats: (c0 << 32) | r0, the tile's origin in the  */
                           /* stored matrix (tensor-map coordinates)                    */
    int32_t ld, ld2;       /* FP64 leading dimension; mixed formats: tensor map index   */
    int16_t nr, nc;
    int32_t in0, out0, in1, out1;
    uint8_t k_in0, k_out0, k_in1, k_out1;
};
static_assert(sizeof(Tile) == 48, "tile descriptor layout");

/* One tile of the multi-density tensor-core kernel: rows [r0, r0 + nr),
 * columns [c0, c0 + nc) (nr, nc <= 128) of a stored matrix in its mixed
 * arena (a2: element offset of the tile origin, ld2: leading dimension),
 * the same optional products as Tile, the tile's power-of-two scale
 * exponents (128 row and 128 column int8 values at scales + 256 * index),
 * the byte offset of its pre-computed bf16 slices in the slice arena
 * (4 slices x ceil(nc / 64) column blocks x ceil(nr / 8) swizzle atoms of
 * 1 KB, in that order; in a batch plan, the slices' device address), and
 * in a batch plan the index of the structure whose vectors it uses. */
struct TileM {
    uint64_t a2;
    uint64_t s_off;
    int32_t ld2;
    int16_t nr, nc;
    int32_t in0, out0, in1, out1;
    uint8_t k_in0, k_out0, k_in1, k_out1;
    int32_t fmt;
    int32_t mol;
    int32_t pad_;
};
static_assert(sizeof(TileM) == 56, "multi-density tile descriptor layout");
constexpr int kMmaRows = 128;      /* rows and columns of a TileM */
constexpr int kMmaMinVec = 2;      /* densities per launch from which the tensor-core kernel runs */

/* One product of the launch plan (a stored matrix, its location in the
 * arenas and the vector ranges of its N and T sides), kept so that the tile
 * plan can be rebuilt with other tile shapes (autotuning). */
struct PlanRec {
    uint64_t a, a2;
    int ld, ld2, map, fmt;
    int nrow, ncol;
    int in0, out0, in1, out1;
    uint8_t kin0, kout0, kin1, kout1;
};

/* Launch choices of one structure, picked by the autotuner
 * (H2ERI_gpu_autotune) or left at their defaults. */
struct TuneCfg {
    int chunk_rows = 512;      /* rows per tile of the single-density tile kernels (64..512), or 0: */
                               /* per range, the tallest that gives two waves of CTAs              */
    int tiles_per_cta = 2;     /* mixed single-density kernel: tiles per CTA (1 or 2)               */
    int nf_concurrent = 1;     /* near-field lanes on their own streams (1) or one stream (0)       */
    int mma_min_vec = 2;       /* densities per launch from which the tensor-core kernel runs       */
    int mma_grid_div = 1;      /* tensor-core launches use n_SM / mma_grid_div CTAs                  */
    int persist = 0;           /* mixed single-density path: one persistent launch (1) or a launch  */
                               /* per range on the stream lanes (0)                                 */
};

/* One work item of the persistent mixed-mode kernel: a tile of the plan for
 * one vector, the range (group) whose completion counter it advances, the
 * range that must be complete before it reads its input vectors (-1: none)
 * and the storage format of its matrix. */
struct PItem {
    int32_t tile;
    int16_t group, dep;
    int16_t v, fmt;
    int32_t pad_;
};
static_assert(sizeof(PItem) == 16, "work item layout");

/* Work list of the persistent kernel for one vector count: the items in
 * claim order, the item count of every range, and the control words
 * (ticket, abort flag, per-range completion counters), zeroed before each
 * launch. */
struct PxPlan {
    PItem *items = nullptr;
    int n_items = 0;
    int *gneed = nullptr;
    int n_groups = 0;
    int *ctl = nullptr;
    int ctl_ints = 0;
    int nvec = 0;
    int grid = 0;
    double sim_ms = 0.0;   /* makespan of the host schedule simulation */
};

/* Storage formats of the stored matrices. */
enum MatFmt : int {
    FMT_F64 = 0,    /* double                                               */
    FMT_F32 = 1,    /* float (coupling and near-field blocks, mixed mode)   */
    FMT_F32X2 = 2   /* float pair hi + lo, value = hi + lo (bases, mixed)   */
};

/* One matrix to copy into the mixed arenas when mixed mode is first used. */
struct PackItem {
    const double *src;
    int nrow, ncol, lds;  /* source matrix (row-major) */
    int trans;            /* 1: store the ncol x nrow transpose */
    int fmt;              /* FMT_F32 or FMT_F32X2 */
    size_t off;           /* element offset in the float (F32) or float2 (F32X2) arena */
    int ld;               /* leading dimension of the stored matrix */
};

constexpr int kChunkRows = 512;    /* rows per tile (CTA), a multiple of 64   */
constexpr int kTileCols = 128;
constexpr int kTileThreads = 256;

struct VecArgs {
    double *base[VK_COUNT];
    long long stride[VK_COUNT];
};

#ifdef __CUDACC__
/* Element off of vector v of a vector space (device code). */
__device__ __forceinline__ double *vec_ptr(const VecArgs &va, uint8_t kind, int off, int v)
{
    return va.base[kind] + (long long)v * va.stride[kind] + off;
}
#endif

/* One structure of a batch plan: its vector spaces and its number of
 * densities. */
struct BatchMol {
    VecArgs va;
    int nvec;
    int pad_;
};

struct Range {
    int first = 0, count = 0;
    bool pair = false;     /* mixed mode: matrices of this range are float pairs */
    int lane = 0;          /* near field: the stream (independent stage chain) it runs on */
};
constexpr int kNfLanes = 2;   /* near-field lanes: float-pair blocks, then groups of single-float blocks */

/* Device copy of one H2 representation plus the launch plan. */
struct DevRep {
    int device = -1;
    /* fingerprint of the host structure this was built from */
    int krnl = 0, n_node = 0, num_bf = 0, n_B = 0, n_D = 0;
    const void *fp_U = nullptr, *fp_B = nullptr, *fp_D = nullptr;
    /* blocks */
    double *arena = nullptr;
    size_t arena_elems = 0;
    float *arena32 = nullptr;         /* B and D blocks, mixed mode */
    void *tmaps = nullptr;            /* one 128-byte tensor map per mixed-arena matrix (TMA loads) */
    unsigned *err_flag = nullptr;     /* mapped host word: nonzero after a kernel gave up a bounded wait */
    unsigned *err_flag_dev = nullptr; /* its device address */
    float2 *arena32x2 = nullptr;      /* U bases as hi/lo pairs, mixed mode */
    size_t arena32_elems = 0, arena32x2_elems = 0;
    std::vector<PackItem> mixed_items;
    double alg_bytes_matrix_mixed = 0.0;
    size_t bytes_U = 0, bytes_B = 0, bytes_D = 0;
    /* plan */
    Tile *tiles = nullptr;
    int n_tiles = 0;
    std::vector<Tile> tiles_host;   /* host copy of the tile plan (batch plans) */
    std::vector<Range> fwd;     /* deepest level first */
    std::vector<Range> bwd;     /* shallowest level first */
    std::vector<Range> mid;     /* coupling blocks, stages 1..3 */
    std::vector<Range> den;     /* near field, stages 1..3 (diagonal-pair, then single-float range per stage) */
    int rank_total = 0, lr_total = 0;
    /* algorithmic bytes / flops of one matvec (per vector), for reports */
    double alg_bytes_matrix = 0.0, alg_bytes_vec = 0.0, alg_flops = 0.0;
    /* J assembly maps */
    int *unc_map = nullptr;      /* krnl entries: (D index << 1) | off-diagonal flag */
    int *con_map = nullptr;      /* num_bf^2 entries: (y index << 1) | diagonal flag, or -1 */
    /* work space */
    double *work = nullptr;      /* [Y0 | Y1 | T] regions, nvec_cap vectors each */
    int nvec_cap = 0;
    double *xbuf = nullptr, *ybuf = nullptr;   /* matvec staging, nvec_cap vectors */
    double *dbuf = nullptr, *jbuf = nullptr;   /* density / J staging, nden_cap matrices */
    int nden_cap = 0;
    cudaStream_t s_main = nullptr, s_aux = nullptr;   /* s_aux: near-field lane 0 */
    cudaStream_t s_nf[kNfLanes] = {nullptr};          /* near-field lanes 1.. (s_nf[0] unused) */
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_zero = nullptr, ev_done = nullptr;
    cudaEvent_t ev_nf[kNfLanes] = {nullptr};
    cudaEvent_t ev_bfork = nullptr, ev_bjoin = nullptr;   /* batched builds: fork from / join to the caller */
    cudaEvent_t ev_t[8] = {nullptr};
    float last_ms[5] = {0, 0, 0, 0, 0};   /* fwd, mid, bwd, den, total */
    int precision = 0;
    double *noalloc_work = nullptr;   /* device address of the fixed scratch array (matvec without allocation) */
    /* multi-density tensor-core plan (mixed mode): 128 x 128 tiles with the
     * same phases as the tile plan, their scale exponents and slices */
    TileM *mtiles = nullptr;
    int8_t *mscales = nullptr;
    unsigned char *mslices = nullptr;
    size_t mslice_bytes = 0;
    int n_mtiles = 0;
    std::vector<TileM> mtiles_host;
    std::vector<Range> mfwd, mmid, mbwd, mden;
    int mma_levels = 5;          /* slice levels of the multi-density kernel (4 or 5) */
    int n_sm = 0;
    PxPlan px;                   /* persistent kernel's work list (mixed mode, built on first use) */
    /* the products behind every range of fwd, mid, bwd, den (same order), for re-planning */
    std::vector<std::vector<PlanRec>> rec_fwd, rec_mid, rec_bwd, rec_den;
    TuneCfg cfg;                 /* launch choices (autotuned or default) */
    void *kstate = nullptr;      /* exchange plan and buffers, built on first use */
    double k_work_bytes = 0.0;   /* exchange work-tensor budget, 0 = from free memory */
};

}  // namespace h2g

#endif
