/*
 * GPU H2 apply: device representation, launch plan and the kernels of
 * the hot path (H2P-ERI src/H2ERI_matvec.c:882-957 and
 * src/H2ERI_build_Coulomb.c:26-152).
 *
 * Every stored matrix (nested basis U, coupling block B, near-field block D,
 * or one factor of a low-rank B/D) is cut into tiles of up to kChunkRows (512)
 * rows by kTileCols (128) columns. One CTA runs one tile (FP64) or two
 * (mixed formats) and performs the products the reference does for a block:
 *   upward sweep   (src/H2ERI_matvec.c:93-175)   T-product with U
 *   B intermediate (src/H2ERI_matvec.c:299-407)  N and T products (bi-GEMV)
 *   downward sweep (src/H2ERI_matvec.c:663-757)  N-product with U
 *   near field     (src/H2ERI_matvec.c:572-660)  N (diagonal) or N and T
 * Partial sums go to the output vectors with FP64 atomics, replacing the
 * reference's per-thread copies and reductions. The children of a node keep
 * their coefficient segments next to each other, so a non-leaf U reads or
 * writes one contiguous slice. The near field depends only on x and runs on
 * a second stream concurrently with the tree sweeps.
 */
#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <queue>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda.h>

#include "h2eri_gb300.h"
#include "h2g_device.cuh"
#include "h2g_farith.cuh"
#include "h2g_gpu_stats.h"
#include "h2g_gpu_api.h"

namespace h2g {

/* ======================================================================== */
/* Error state                                                               */
/* ======================================================================== */

static thread_local std::string t_last_error;

void set_error(const std::string &msg) { t_last_error = msg; }

#define CUDA_TRY(call)                                                                           \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                      \
            return 10;                                                                           \
        }                                                                                        \
    } while (0)

/* ======================================================================== */
/* Kernels                                                                   */
/* ======================================================================== */


/* Column owned by lane `lane` in slot k (0..3) of a 128-column tile strip. */
template <int FMT>
__device__ __forceinline__ int lane_col(int lane, int k)
{
    if (FMT == FMT_F32) return 4 * lane + k;
    return (k < 2) ? 2 * lane + k : 64 + 2 * lane + (k - 2);
}

/* ---- shared-memory staging with cp.async ---- */
constexpr int kStageBytes = 32768;
constexpr int kStages = 3;
constexpr size_t kTileSmem = (size_t)kStageBytes * kStages;
constexpr size_t kTileSmemLaunch = kTileSmem + 1024;   /* + slack to align the TMA destinations */

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

/* ---- TMA (tensor copies) and mbarriers, FP32 formats ---- */
constexpr int kTmaBoxBytes = 128;              /* inner box extent: one 128-byte swizzle span */
constexpr long long kWaitCycles = 2000000000LL; /* bound of every mbarrier wait (~1 s) */

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}
/* Wait for phase `parity` of an mbarrier, giving up after `limit` cycles. */
__device__ __noinline__ bool mbar_wait(unsigned bar, unsigned parity, long long limit = kWaitCycles)
{
    if (mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try(bar, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}
/* 2-D tensor copy of one box into shared memory, completing on bar. The
 * stored matrices stream through L2 once per matvec, so the copies are marked
 * evict-first: they then do not push out the small vectors that the FP64
 * output atomics work on (measured 0.438 -> 0.418 ms per C30H62 J build). */
__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap *map, int x, int y, unsigned bar)
{
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, %3}], [%4], %5;"
                 ::"r"(dst), "l"(map), "r"(x), "r"(y), "r"(bar), "l"(pol)
                 : "memory");
}

template <int FMT> struct FmtInfo;
template <> struct FmtInfo<FMT_F64> { static constexpr int ebytes = 8; };
template <> struct FmtInfo<FMT_F32> { static constexpr int ebytes = 4; };
template <> struct FmtInfo<FMT_F32X2> { static constexpr int ebytes = 8; };

/* Issue the copies of one stage: rows [row0, row0 + SR) of the tile, all
 * kTileCols columns, into a dense SR x (kTileCols * ebytes) smem block. Rows
 * at or beyond nr that a warp with rows inside the tile reads, and columns
 * beyond the tile, are zero-filled. In the FP32 formats the 16-byte chunk cc
 * of stage row r goes to chunk position cc ^ (r & 31) of that row, so that
 * 32 lanes reading one chunk column of 32 rows hit distinct banks (the
 * lane-per-row N side) as well as 32 lanes reading one row. */
template <int FMT>
__device__ __forceinline__ void issue_stage(unsigned char *buf, const unsigned char *base, size_t ld_bytes, int row0,
                                            int nr, int nc_bytes16, int tid)
{
    constexpr int RB = kTileCols * FmtInfo<FMT>::ebytes;   /* bytes per stage row */
    constexpr int CPR = RB / 16;                            /* 16-byte chunks per row */
    constexpr int NCH = kStageBytes / 16;
    /* rows never read (their warps have no row in the tile) are not copied:
     * FP64 reads 8-row blocks per warp, the FP32 formats 32-row groups */
    constexpr int RGRP = (FMT == FMT_F64) ? kStageBytes / RB / 8 : 32;
#pragma unroll
    for (int j = 0; j < NCH / kTileThreads; j++) {
        const int c = tid + j * kTileThreads;
        const int row = c / CPR, cc = c - row * CPR;
        const int grow = row0 + row;
        if (row0 + (row / RGRP) * RGRP >= nr) continue;
        const int pos = (FMT == FMT_F64) ? cc : (cc ^ (row & 31));
        int valid = 0;
        const unsigned char *src = base;
        if (grow < nr) {
            valid = min(16, max(0, nc_bytes16 - cc * 16));
            if (valid > 0) src = base + (size_t)grow * ld_bytes + cc * 16;
        }
        cp_async16(buf + (size_t)row * RB + pos * 16, src, valid);
    }
}

/* Row partials of R rows per warp (R = 8 or 4) reduced across the warp by
 * recursive halving; returns the value of row `halving_row_R(lane)` on the
 * lanes that finish with a full sum. */
template <int R>
__device__ __forceinline__ int halving_row_R(int lane)
{
    if (R == 8) return ((lane & 16) ? 4 : 0) + ((lane & 8) ? 2 : 0) + ((lane & 4) ? 1 : 0);
    return ((lane & 16) ? 2 : 0) + ((lane & 8) ? 1 : 0);
}
template <int R>
__device__ __forceinline__ bool halving_owner(int lane)
{
    return (R == 8) ? ((lane & 3) == 0) : ((lane & 7) == 0);
}

template <int R>
__device__ __forceinline__ double reduceR_f64(double *s, int lane)
{
    const bool b16 = lane & 16, b8 = lane & 8;
    if constexpr (R == 8) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            double send = b16 ? s[k] : s[k + 4];
            double keep = b16 ? s[k + 4] : s[k];
            s[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
        }
#pragma unroll
        for (int k = 0; k < 2; k++) {
            double send = b8 ? s[k] : s[k + 2];
            double keep = b8 ? s[k + 2] : s[k];
            s[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
        }
        const bool b4 = lane & 4;
        double send = b4 ? s[0] : s[1];
        double val = (b4 ? s[1] : s[0]) + __shfl_xor_sync(0xffffffffu, send, 4);
        val += __shfl_xor_sync(0xffffffffu, val, 2);
        val += __shfl_xor_sync(0xffffffffu, val, 1);
        return val;
    } else {
#pragma unroll
        for (int k = 0; k < 2; k++) {
            double send = b16 ? s[k] : s[k + 2];
            double keep = b16 ? s[k + 2] : s[k];
            s[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
        }
        double send = b8 ? s[0] : s[1];
        double val = (b8 ? s[1] : s[0]) + __shfl_xor_sync(0xffffffffu, send, 8);
        val += __shfl_xor_sync(0xffffffffu, val, 4);
        val += __shfl_xor_sync(0xffffffffu, val, 2);
        val += __shfl_xor_sync(0xffffffffu, val, 1);
        return val;
    }
}

/* FP64 tile kernel. One CTA per (vector, tile). A tile is a chunk of up to
 * kChunkRows rows and kTileCols columns. The chunk streams through a
 * kStages-deep ring of 32 KB shared-memory stages filled with cp.async
 * (16-byte copies, any leading dimension, zero fill past the tile edge), so
 * the next stages are in flight while the current one is multiplied. A stage
 * holds SR = 32 rows of doubles; warp w multiplies rows [w*SR/8, (w+1)*SR/8)
 * and each lane owns 4 columns (lane_col). N-side row sums are added per
 * stage; T-side column sums stay in registers over the whole chunk and are
 * added once (few atomics per coefficient). FP64 FMAs and FP64 reductions
 * (FMT_F64 only; the FP32 formats of the mixed mode run k_tile_mx). */
template <int FMT>
__global__ void __launch_bounds__(kTileThreads, 2)
k_tile(const Tile *__restrict__ tiles, const void *__restrict__ arena_v, const __grid_constant__ VecArgs va)
{
    constexpr int EB = FmtInfo<FMT>::ebytes;
    constexpr int SR = kStageBytes / (kTileCols * EB);   /* rows per stage   */
    constexpr int RW = SR / 8;                            /* rows per warp    */
    constexpr int RB = kTileCols * EB;                    /* bytes per row    */
    static_assert(FMT == FMT_F64, "the mixed formats use k_tile_mx");
    extern __shared__ __align__(128) unsigned char stage_raw[];

    /* the vector index runs fastest: the CTAs of one tile for several
     * densities run back to back and share the tile through L2 */
    const Tile t = tiles[blockIdx.y];
    const int v = blockIdx.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool opN = t.k_out0 != VK_NONE, opT = t.k_out1 != VK_NONE;
    const int nr = t.nr, nc = t.nc;
    const int nstage = (nr + SR - 1) / SR;
    const unsigned char *base = reinterpret_cast<const unsigned char *>(arena_v) + (size_t)t.a * EB;   /* FP64 */
    const size_t ld_bytes = (size_t)t.ld * EB;
    const int nc_bytes16 = ((nc * EB) + 15) & ~15;

    /* prologue: first two stages in flight */
    if (FMT == FMT_F64) {
        issue_stage<FMT>(stage_raw, base, ld_bytes, 0, nr, nc_bytes16, tid);
        cp_async_commit();
        if (nstage > 1) issue_stage<FMT>(stage_raw + kStageBytes, base, ld_bytes, SR, nr, nc_bytes16, tid);
        cp_async_commit();
    }

    double *out0 = opN ? vec_ptr(va, t.k_out0, t.out0, v) : nullptr;
    bool ok[4];
#pragma unroll
    for (int k = 0; k < 4; k++) ok[k] = lane_col<FMT>(lane, k) < nc;
    /* byte offsets of this lane's two 16-byte pieces inside a stage row */
    const int offA = (FMT == FMT_F32) ? 16 * lane : 16 * lane;
    const int offB = 512 + 16 * lane;   /* used by the 8-byte formats only */

    if (FMT == FMT_F64) {
        double xv[4] = {0.0, 0.0, 0.0, 0.0};
        if (opN) {
            const double *in0 = vec_ptr(va, t.k_in0, t.in0, v);
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (ok[k]) xv[k] = in0[lane_col<FMT>(lane, k)];
        }
        const double *in1 = opT ? vec_ptr(va, t.k_in1, t.in1, v) : nullptr;
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for (int k = 0; k < nstage; k++) {
            cp_async_wait1();
            __syncthreads();
            if (k + 2 < nstage)
                issue_stage<FMT>(stage_raw + ((k + 2) % kStages) * kStageBytes, base, ld_bytes, (k + 2) * SR, nr,
                                 nc_bytes16, tid);
            cp_async_commit();
            const unsigned char *buf = stage_raw + (k % kStages) * kStageBytes;
            const int r0 = k * SR + warp * RW;
            if (r0 >= nr) continue;   /* no row of this warp in the tile (warp-uniform) */
            double a[RW][4];
#pragma unroll
            for (int i = 0; i < RW; i++) {
                const unsigned char *row = buf + (warp * RW + i) * RB;
                const double2 pa = *reinterpret_cast<const double2 *>(row + offA);
                const double2 pb = *reinterpret_cast<const double2 *>(row + offB);
                a[i][0] = pa.x; a[i][1] = pa.y; a[i][2] = pb.x; a[i][3] = pb.y;
            }
            if (opN) {
                double sr[RW];
#pragma unroll
                for (int i = 0; i < RW; i++) sr[i] = a[i][0] * xv[0] + a[i][1] * xv[1] + a[i][2] * xv[2] + a[i][3] * xv[3];
                const double val = reduceR_f64<RW>(sr, lane);
                const int row = r0 + halving_row_R<RW>(lane);
                if (halving_owner<RW>(lane) && row < nr) atomicAdd(out0 + row, val);
            }
            if (opT) {
#pragma unroll
                for (int i = 0; i < RW; i++) {
                    const double x1 = (r0 + i < nr) ? in1[r0 + i] : 0.0;
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[c] += a[i][c] * x1;
                }
            }
        }
        if (opT) {
            /* reduce over the warps through the last stage's slot (no copy is pending into it) */
            __syncthreads();
            double (*red)[kTileCols] =
                reinterpret_cast<double (*)[kTileCols]>(stage_raw + ((nstage - 1) % kStages) * kStageBytes);
#pragma unroll
            for (int c = 0; c < 4; c++) red[warp][lane_col<FMT>(lane, c)] = acc[c];
            __syncthreads();
            double *out1 = vec_ptr(va, t.k_out1, t.out1, v);
            for (int c = tid; c < nc; c += kTileThreads) {
                double sum = 0.0;
#pragma unroll
                for (int w = 0; w < 8; w++) sum += red[w][c];
                atomicAdd(out1 + c, sum);
            }
        }
        return;
    }

}

/* Shared memory of k_tile_mx (dynamic, laid out here): the stage ring first
 * (TMA destinations with the 128-byte swizzle must start on 1024-byte
 * boundaries; the kernel checks and refuses otherwise), then the N-side box
 * partials of the stages in flight, the split inputs of both tiles, the
 * stage mbarriers and the slot and row-group counters. Two CTAs fit in one
 * SM (2 x (112 KB + 1 KB reserved) of 228 KB). */
struct MxInputs {
    float x0h[kTileCols], x0l[kTileCols], x1h[kChunkRows], x1l[kChunkRows];
};
struct MxSmem {
    unsigned char ring[kStages][kStageBytes];
    float2 npart[kStages][256];
    MxInputs sx[2];
    unsigned long long full[kStages];
    int slot_cnt[kStages];
    int grp_cnt[kStages][2];
    int dead;
};
constexpr size_t kMxSmem = (sizeof(MxSmem) + 127) & ~size_t(127);

/* One stage of a tile in the mixed-mode kernels (FP32 formats): the stage
 * in ring slot `slot` holds rows [k SR, k SR + SR) of tile t (SR = 64 rows
 * of single floats or 32 rows of float pairs). N side: out0 += A x0 over the
 * stage's rows (lane per row, one box per warp, box partials merged by the
 * last warp of the row group); T side: the column sums over the stage's rows
 * are folded into the warp's float-pair accumulators ch / cl, which are
 * reduced and added to out1 after the tile's last stage (`last`). Products
 * are accumulated in anchored chains (h2g_farith.cuh). */
template <int FMT>
__device__ __forceinline__ void mx_stage(MxSmem &sm, int slot, const Tile &t, const MxInputs &X, int k, bool last,
                                         double *out0, double *out1, float2 (&ch)[2], float2 (&cl)[2])
{
    constexpr int EB = FmtInfo<FMT>::ebytes;
    constexpr int SR = kStageBytes / (kTileCols * EB);   /* rows per stage: 64 or 32   */
    constexpr int RB = kTileCols * EB;                    /* bytes per stage row        */
    constexpr int NB = RB / kTmaBoxBytes;                 /* boxes per stage: 4 or 8    */
    constexpr int BOXB = SR * kTmaBoxBytes;               /* bytes per box              */
    constexpr int NG = SR / 32;                           /* N-side 32-row groups       */
    constexpr int NCG = 8 / NG;                           /* boxes (warps) per group    */
    static_assert(NCG == NB, "one box per N-side warp");
    constexpr int TC = (FMT == FMT_F32) ? 4 : 8;          /* T side: chunks per warp row */
    constexpr int TL = 32 / TC;                           /* T side: row lanes          */
    constexpr int TR = SR / TL;                           /* T side: rows per lane      */
    static_assert(TR == 8, "T-side lane layout");
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ng = warp % NG, cg = warp / NG;
    const int tb = (FMT == FMT_F32) ? warp >> 1 : warp;                 /* T side: box      */
    /* T side: chunk and row lane. A 16-byte load is served per quarter warp
     * (8 lanes), which must hit 8 different chunk positions: with 4 chunks
     * per row lane (single floats) a quarter warp takes rows r and r + 4,
     * whose swizzles map the 4 chunks to the two halves of the line. */
    const int tq = ((FMT == FMT_F32) ? (warp & 1) * 4 : 0) + lane % TC;
    const int trl = (FMT == FMT_F32) ? (lane >> 3) + 4 * ((lane >> 2) & 1) : lane / TC;
    const bool opN = t.k_out0 != VK_NONE, opT = t.k_out1 != VK_NONE;
    const unsigned char *buf = sm.ring[slot];
    const int nr = t.nr;
    if (opN && k * SR + ng * 32 < nr) {
        /* the lane's row over one box: two anchored chains (even and odd
         * columns), bounded by their own sums |a| |xh| */
        const int rr = ng * 32 + lane;
        const unsigned char *rowp = buf + cg * BOXB + rr * kTmaBoxBytes;
        float4 q[8];
#pragma unroll
        for (int j = 0; j < 8; j++) q[j] = *reinterpret_cast<const float4 *>(rowp + 16 * (j ^ (rr & 7)));
        float2 b0 = make_float2(0.f, 0.f), b1 = b0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int cc = cg * 8 + j;
            if (FMT == FMT_F32) {
                const float4 xh = *reinterpret_cast<const float4 *>(X.x0h + 4 * cc);
                b0 = pk_fma(pk_abs(make_float2(q[j].x, q[j].y)), pk_abs(make_float2(xh.x, xh.y)), b0);
                b1 = pk_fma(pk_abs(make_float2(q[j].z, q[j].w)), pk_abs(make_float2(xh.z, xh.w)), b1);
            } else {
                const float2 xh = *reinterpret_cast<const float2 *>(X.x0h + 2 * cc);
                if (j & 1) b1 = pk_fma(pk_abs(make_float2(q[j].x, q[j].y)), pk_abs(xh), b1);
                else b0 = pk_fma(pk_abs(make_float2(q[j].x, q[j].y)), pk_abs(xh), b0);
            }
        }
        /* two chains per half on one anchor (bounded by both): their high
         * parts are multiples of one ulp below 2^(k-2) and add exactly */
        const float2 s0 = anchor2(pk_add(b0, b1)), z = make_float2(0.f, 0.f);
        float2 sa = s0, sb = s0, la1 = z, la2 = z, lb1 = z, lb2 = z;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int cc = cg * 8 + j;
            if (FMT == FMT_F32) {
                const float4 xh = *reinterpret_cast<const float4 *>(X.x0h + 4 * cc);
                const float4 xl = *reinterpret_cast<const float4 *>(X.x0l + 4 * cc);
                pk_aacc1(sa, la1, la2, make_float2(q[j].x, q[j].y), make_float2(xh.x, xh.y), make_float2(xl.x, xl.y));
                pk_aacc1(sb, lb1, lb2, make_float2(q[j].z, q[j].w), make_float2(xh.z, xh.w), make_float2(xl.z, xl.w));
            } else {
                const float2 xh = *reinterpret_cast<const float2 *>(X.x0h + 2 * cc);
                const float2 xl = *reinterpret_cast<const float2 *>(X.x0l + 2 * cc);
                if (j & 1) pk_aacc2(sb, lb1, lb2, make_float2(q[j].x, q[j].y), make_float2(q[j].z, q[j].w), xh, xl);
                else pk_aacc2(sa, la1, la2, make_float2(q[j].x, q[j].y), make_float2(q[j].z, q[j].w), xh, xl);
            }
        }
        const float2 hi = pk_add(pk_sub(sa, s0), pk_sub(sb, s0));   /* exact */
        const float2 lo = pk_add(pk_add(la1, la2), pk_add(lb1, lb2));
        float h = hi.x, l = lo.x;
        dfadd(h, l, hi.y, lo.y);
        sm.npart[slot][cg * SR + rr] = make_float2(h, l);
    }

    if (opT) {
        /* the lane's chunk over rows trl + TL i of the stage: anchored
         * chains per column, folded into the tile's float-pair column
         * sums once per stage. Rows past the tile have zero inputs. */
        float4 q[TR];
#pragma unroll
        for (int i = 0; i < TR; i++) {
            const int rr = trl + TL * i;
            q[i] = *reinterpret_cast<const float4 *>(buf + tb * BOXB + rr * kTmaBoxBytes + 16 * (tq ^ (rr & 7)));
        }
        const float *x1h = X.x1h + k * SR + trl, *x1l = X.x1l + k * SR + trl;
        float2 b0 = make_float2(0.f, 0.f), b1 = b0;
#pragma unroll
        for (int i = 0; i < TR; i++) {
            const float2 xa = bcast(fabsf(x1h[TL * i]));
            if (FMT == FMT_F32) {
                b0 = pk_fma(pk_abs(make_float2(q[i].x, q[i].y)), xa, b0);
                b1 = pk_fma(pk_abs(make_float2(q[i].z, q[i].w)), xa, b1);
            } else {
                b0 = pk_fma(pk_abs(make_float2(q[i].x, q[i].y)), xa, b0);
            }
        }
        if (FMT == FMT_F32) {
            const float2 s0 = anchor2(b0), s1 = anchor2(b1), z = make_float2(0.f, 0.f);
            float2 sa = s0, sb = s1, la1 = z, la2 = z, lb1 = z, lb2 = z;
#pragma unroll
            for (int i = 0; i < TR; i++) {
                const float2 xh = bcast(x1h[TL * i]), xl = bcast(x1l[TL * i]);
                pk_aacc1(sa, la1, la2, make_float2(q[i].x, q[i].y), xh, xl);
                pk_aacc1(sb, lb1, lb2, make_float2(q[i].z, q[i].w), xh, xl);
            }
            pk_dfadd(ch[0], cl[0], pk_sub(sa, s0), pk_add(la1, la2));
            pk_dfadd(ch[1], cl[1], pk_sub(sb, s1), pk_add(lb1, lb2));
        } else {
            /* two chains over alternate rows on one anchor: their high
             * parts are multiples of one ulp below 2^(k-2), so they add
             * exactly */
            const float2 s0 = anchor2(b0), z = make_float2(0.f, 0.f);
            float2 sa = s0, sb = s0, la1 = z, la2 = z, lb1 = z, lb2 = z;
#pragma unroll
            for (int i = 0; i < TR; i += 2) {
                const float2 xh0 = bcast(x1h[TL * i]), xl0 = bcast(x1l[TL * i]);
                const float2 xh1 = bcast(x1h[TL * (i + 1)]), xl1 = bcast(x1l[TL * (i + 1)]);
                pk_aacc2(sa, la1, la2, make_float2(q[i].x, q[i].y), make_float2(q[i].z, q[i].w), xh0, xl0);
                pk_aacc2(sb, lb1, lb2, make_float2(q[i + 1].x, q[i + 1].y), make_float2(q[i + 1].z, q[i + 1].w), xh1,
                         xl1);
            }
            pk_dfadd(ch[0], cl[0], pk_add(pk_sub(sa, s0), pk_sub(sb, s0)),
                     pk_add(pk_add(la1, la2), pk_add(lb1, lb2)));
        }
        if (last) {
            /* tile done: reduce the column sums over the row lanes */
#pragma unroll
            for (int off = TC; off < 32; off <<= 1)
#pragma unroll
                for (int j = 0; j < (FMT == FMT_F32 ? 2 : 1); j++) {
                    const float2 oh = make_float2(__shfl_xor_sync(0xffffffffu, ch[j].x, off),
                                                  __shfl_xor_sync(0xffffffffu, ch[j].y, off));
                    const float2 ol = make_float2(__shfl_xor_sync(0xffffffffu, cl[j].x, off),
                                                  __shfl_xor_sync(0xffffffffu, cl[j].y, off));
                    pk_dfadd(ch[j], cl[j], oh, ol);
                }
            if (trl == 0) {
                if (FMT == FMT_F32) {
                    const int c = tb * 32 + tq * 4;
                    if (c < t.nc) atomic_add_pair(out1 + c, ch[0].x, cl[0].x);
                    if (c + 1 < t.nc) atomic_add_pair(out1 + c + 1, ch[0].y, cl[0].y);
                    if (c + 2 < t.nc) atomic_add_pair(out1 + c + 2, ch[1].x, cl[1].x);
                    if (c + 3 < t.nc) atomic_add_pair(out1 + c + 3, ch[1].y, cl[1].y);
                } else {
                    const int c = tb * 16 + tq * 2;
                    if (c < t.nc) atomic_add_pair(out1 + c, ch[0].x, cl[0].x);
                    if (c + 1 < t.nc) atomic_add_pair(out1 + c + 1, ch[0].y, cl[0].y);
                }
            }
        }
    }

    __syncwarp();
    if (opN) {
        /* the last warp of the row group merges the group's box partials */
        int last = 0;
        if (lane == 0) {
            __threadfence_block();
            last = atomicAdd(&sm.grp_cnt[slot][ng], 1) == NCG - 1;
        }
        if (__shfl_sync(0xffffffffu, last, 0)) {
            __threadfence_block();
            const int rr = ng * 32 + lane, grow = k * SR + rr;
            if (grow < nr) {
                const float2 *P = sm.npart[slot];
                float h = P[rr].x, l = P[rr].y;
#pragma unroll
                for (int q = 1; q < NCG; q++) dfadd(h, l, P[q * SR + rr].x, P[q * SR + rr].y);
                atomic_add_pair(out0 + grow, h, l);
            }
            if (lane == 0) sm.grp_cnt[slot][ng] = 0;
        }
        __syncwarp();
    }
}

/* Mixed-mode tile kernel (FP32 formats), two tiles per CTA. Stages arrive
 * by TMA as NB swizzled boxes of SR rows x 128 bytes (16-byte chunk q of box
 * row r at q ^ (r & 7)) into a kStages-deep ring that runs across both
 * tiles; both tiles' input slices are split into float pairs up front. CTA
 * (v, y) of a launch with G CTAs per vector takes tiles y and y + G.
 *
 * The warps never wait for one another inside the loop, only for their
 * data: the last warp to finish with a ring slot (a shared counter) reloads
 * it with the stage kStages ahead, so up to kStages stages are in flight and
 * a warp that is done with a short stage moves on to the next one.
 *   N side: lane per row; warp (ng, cg) takes rows [32 ng, 32 ng + 32) of a
 *     stage over box cg; the box partials of a row group are merged by the
 *     last of its warps to finish (a second counter) and added to out0.
 *   T side: warp w owns a strip of 16-byte chunks of every row (4 chunks of
 *     box w / 2 for single floats, all 8 chunks of box w for pairs); its
 *     lanes split the strip's chunks and the stage's rows, so the column
 *     sums of a tile are reduced inside the warp (shuffles) and added once.
 * Products are accumulated in anchored chains (h2g_farith.cuh): per lane, one
 * chain per box of a row (N) or per column over the lane's rows of a stage
 * (T), anchored on its own bound sum |a| |xh|, so the only error that
 * matters is the storage rounding of the matrix (2^-24 relative for FMT_F32,
 * ~2^-48 for FMT_F32X2; plain FP32 FMA chains roughly double it, measured
 * 1.2e-8 vs 5e-9 on C10H22). Every output element is converted to FP64 once
 * and added with FP64 atomics. */
template <int FMT, bool BATCH>
__global__ void __launch_bounds__(kTileThreads, 2)
k_tile_mx(const Tile *__restrict__ tiles, int n_tiles, const __grid_constant__ VecArgs va,
          const CUtensorMap *__restrict__ maps, unsigned *err, const BatchMol *__restrict__ mols)
{
    /* one structure (BATCH false): va; a batch: each tile's structure index
     * is in its FP64 arena offset, which the mixed kernel never reads. A
     * template parameter, so that the single-structure kernel keeps its
     * registers. */
    auto vp = [&](const Tile &t, uint8_t kind, int off) -> double * {
        if constexpr (BATCH) return vec_ptr(mols[t.a].va, kind, off, (int)blockIdx.x);
        else return vec_ptr(va, kind, off, (int)blockIdx.x);
    };
    constexpr int EB = FmtInfo<FMT>::ebytes;
    constexpr int SR = kStageBytes / (kTileCols * EB);   /* rows per stage: 64 or 32   */
    constexpr int RB = kTileCols * EB;                    /* bytes per stage row        */
    constexpr int NB = RB / kTmaBoxBytes;                 /* boxes per stage: 4 or 8    */
    constexpr int BOXB = SR * kTmaBoxBytes;               /* bytes per box              */
    constexpr int BOXW = kTmaBoxBytes / EB;               /* elements per box row       */
    constexpr int NW = kTileThreads / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    MxSmem &sm = *reinterpret_cast<MxSmem *>(smem_raw);
    volatile int *dead = &sm.dead;

    const int tid = threadIdx.x, lane = tid & 31;
    if (smem_addr(sm.ring) & 1023u) {   /* the same for every thread: nothing has started */
        if (tid == 0) atomicOr(err, 2u);
        return;
    }
    const int G = gridDim.y;   /* vector: blockIdx.x */
    const int ti0 = blockIdx.y, ti1 = blockIdx.y + G;
    const int ntl = ti1 < n_tiles ? 2 : 1;
    const Tile tA = tiles[ti0];
    const Tile tB = tiles[ntl == 2 ? ti1 : ti0];
    const int nsA = (tA.nr + SR - 1) / SR, nsB = ntl == 2 ? (tB.nr + SR - 1) / SR : 0;
    const int S = nsA + nsB;

    auto issue = [&](int g) {   /* one thread: stage g of the CTA's sequence into slot g % kStages */
        const bool b = g >= nsA;
        const Tile &t = b ? tB : tA;
        const int k = b ? g - nsA : g;
        const unsigned bar = smem_addr(&sm.full[g % kStages]);
        const unsigned dst = smem_addr(sm.ring[g % kStages]);
        const CUtensorMap *map = maps + t.ld2;
        const int tc0 = (int)(t.a2 >> 32), tr0 = (int)(t.a2 & 0xffffffffu);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kStageBytes) : "memory");
#pragma unroll
        for (int bx = 0; bx < NB; bx++) tma_load_2d(dst + bx * BOXB, map, tc0 + bx * BOXW, tr0 + k * SR, bar);
    };
    if (tid == 0) {
        for (int i = 0; i < kStages; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&sm.full[i])) : "memory");
            sm.slot_cnt[i] = 0;
            sm.grp_cnt[i][0] = sm.grp_cnt[i][1] = 0;
        }
        sm.dead = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(maps + tA.ld2) : "memory");
        if (ntl == 2)
            asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(maps + tB.ld2) : "memory");
        for (int g = 0; g < kStages && g < S; g++) issue(g);
    }

    /* split the input slices of both tiles */
#pragma unroll
    for (int i = 0; i < 2; i++) {
        if (i >= ntl) break;
        const Tile &t = i ? tB : tA;
        MxInputs &X = sm.sx[i];
        const bool n0 = t.k_out0 != VK_NONE, n1 = t.k_out1 != VK_NONE;
        if (tid < kTileCols) {
            float h = 0.f, l = 0.f;
            if (n0 && tid < t.nc) split(vp(t, t.k_in0, t.in0)[tid], h, l);
            X.x0h[tid] = h; X.x0l[tid] = l;
        }
        if (n1)
            for (int r = tid; r < kChunkRows; r += kTileThreads) {   /* rows >= nr read as zero */
                float h = 0.f, l = 0.f;
                if (r < t.nr) split(vp(t, t.k_in1, t.in1)[r], h, l);
                X.x1h[r] = h; X.x1l[r] = l;
            }
    }
    __syncthreads();   /* inputs, barriers and counters ready; the only CTA-wide barrier */

    float2 ch[2], cl[2];
    int lost = -1;
    for (int g = 0; g < S; g++) {
        const bool b = g >= nsA;
        const Tile &t = b ? tB : tA;
        const MxInputs &X = sm.sx[b ? 1 : 0];
        const int k = b ? g - nsA : g;
        const int slot = g % kStages;
        const bool opN = t.k_out0 != VK_NONE, opT = t.k_out1 != VK_NONE;
        if (!*dead && !mbar_wait(smem_addr(&sm.full[slot]), (unsigned)((g / kStages) & 1))) {
            atomicOr(err, 1u);
            *dead = 1;
            lost = g;
        }
        if (k == 0) ch[0] = ch[1] = cl[0] = cl[1] = make_float2(0.f, 0.f);
        const bool last = k == (b ? nsB : nsA) - 1;
        double *out0 = opN ? vp(t, t.k_out0, t.out0) : nullptr;
        double *out1 = opT ? vp(t, t.k_out1, t.out1) : nullptr;
        mx_stage<FMT>(sm, slot, t, X, k, last, out0, out1, ch, cl);
        /* release the slot; the last warp out reloads it kStages stages ahead */
        if (lane == 0) {
            __threadfence_block();
            if (atomicAdd(&sm.slot_cnt[slot], 1) == NW - 1) {
                sm.slot_cnt[slot] = 0;
                __threadfence_block();
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                if (g + kStages < S && !*dead) issue(g + kStages);
            }
        }
    }
    if (lost >= 0) (void)mbar_wait(smem_addr(&sm.full[lost % kStages]), (unsigned)((lost / kStages) & 1));
}

/* ---- persistent mixed-mode kernel ---- */

/* Shared memory of k_tile_px: the ring, partials and inputs of k_tile_mx
 * first (so the ring keeps its 1024-byte alignment), then the CTA's item
 * window: up to four claimed items (ring indexed by claim order) with their
 * tiles and stage ranges, and the issue state of the stage sequence that
 * runs across items. */
struct PxSmem {
    MxSmem m;
    Tile tl[4];
    PItem it[4];
    int gs[4], ns[4];   /* first stage (CTA sequence) and stage count of each item */
    int n_known;        /* items claimed so far                                    */
    int exhausted;      /* the queue is empty                                      */
    int stage_end;      /* end of the stage sequence of the claimed items          */
    int ip, ip_item;    /* next stage to issue and its item                        */
};
constexpr size_t kPxSmem = (sizeof(PxSmem) + 127) & ~size_t(127);
static_assert(2 * (kPxSmem + 1024) <= 233472, "two persistent CTAs per SM (228 KB, 1 KB reserved per CTA)");
constexpr int kPxDone = 32;                        /* ctl[kPxDone + g]: items of range g done */

__device__ __forceinline__ int ld_acquire_gpu(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

/* Persistent mixed-mode tile kernel (FP32 formats): the whole H2 matvec in
 * one launch. CTAs take items (one tile for one vector) from a queue in a
 * fixed order (ctl[0] is the next ticket) until it is empty; the order is
 * topological for the dependencies between ranges (upward levels, coupling
 * stages, downward levels on the tree chain; the near-field stages on their
 * lanes), so an item waits only for items with smaller tickets. Before an
 * item's input vectors are read, the range it depends on must be complete
 * (ctl[kPxDone + dep] == gneed[dep]); after its last stage, every thread
 * fences its output atomics and thread 0 counts the item in its range.
 *
 * Deadlock freedom: a CTA claims its next item only after the dependency
 * of its current item is met, so each CTA holds at most one item that is
 * still waiting, and that item waits only for smaller tickets; by induction
 * on the smallest unfinished ticket, every item completes. CTAs need not be
 * co-resident (a CTA that has not started holds no ticket). Every wait is
 * bounded: a dependency wait longer than dep_limit cycles sets error bit 4
 * and ctl[1], which makes every other CTA stop waiting, and the results are
 * invalid.
 *
 * The stage ring runs across items: stages of the claimed next item are
 * copied while the current one is multiplied. Input vectors are read
 * through L2 (ld.global.cg): other CTAs of this launch wrote them. */
__global__ void __launch_bounds__(kTileThreads, 2)
k_tile_px(const Tile *__restrict__ tiles, const PItem *__restrict__ items, int n_items,
          const int *__restrict__ gneed, int *ctl, const __grid_constant__ VecArgs va,
          const CUtensorMap *__restrict__ maps, unsigned *err, long long dep_limit)
{
    constexpr int NW = kTileThreads / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PxSmem &ps = *reinterpret_cast<PxSmem *>(smem_raw);
    MxSmem &sm = ps.m;
    volatile int *dead = &sm.dead;
    const int tid = threadIdx.x, lane = tid & 31;
    if (smem_addr(sm.ring) & 1023u) {   /* the same for every thread: nothing has started */
        if (tid == 0) atomicOr(err, 2u);
        return;
    }

    /* thread 0: the next ticket into the item window */
    auto claim = [&]() {
        if (ps.exhausted || *dead) { ps.exhausted = 1; return; }
        const int tk = atomicAdd(&ctl[0], 1);
        if (tk >= n_items) { ps.exhausted = 1; return; }
        const int s = ps.n_known, e = s & 3;
        const PItem it = items[tk];
        ps.it[e] = it;
        ps.tl[e] = tiles[it.tile];
        const int sr = it.fmt == FMT_F32 ? 64 : 32;
        ps.gs[e] = ps.stage_end;
        ps.ns[e] = (ps.tl[e].nr + sr - 1) / sr;
        ps.stage_end += ps.ns[e];
        ps.n_known = s + 1;
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(maps + ps.tl[e].ld2) : "memory");
    };
    /* thread 0: wait until the range item s depends on is complete */
    auto dep_wait = [&](int s) {
        const PItem &it = ps.it[s & 3];
        if (it.dep < 0 || *dead) return;
        const int need = gneed[it.dep];
        const int *ctr = ctl + kPxDone + it.dep;
        if (ld_acquire_gpu(ctr) >= need) return;
        const long long t0 = clock64();
        while (ld_acquire_gpu(ctr) < need) {
            if (ld_acquire_gpu(ctl + 1) != 0) { *dead = 1; return; }
            if (clock64() - t0 > dep_limit) {
                atomicOr(err, 4u);
                atomicExch(ctl + 1, 1);
                *dead = 1;
                return;
            }
            __nanosleep(64);
        }
    };
    /* one thread (no other issuer is active): copies of stages [ip, lim) of
     * the claimed items; the slots of every stage below lim - kStages are free */
    auto issue_upto = [&](int lim) {
        while (ps.ip < ps.stage_end && ps.ip < lim && !*dead) {
            int si = ps.ip_item;
            while (ps.ip >= ps.gs[si & 3] + ps.ns[si & 3]) si++;
            ps.ip_item = si;
            const int e = si & 3, g = ps.ip, k = g - ps.gs[e];
            const Tile &t = ps.tl[e];
            const unsigned bar = smem_addr(&sm.full[g % kStages]);
            const unsigned dst = smem_addr(sm.ring[g % kStages]);
            const CUtensorMap *map = maps + t.ld2;
            const int tc0 = (int)(t.a2 >> 32), tr0 = (int)(t.a2 & 0xffffffffu);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kStageBytes)
                         : "memory");
            if (ps.it[e].fmt == FMT_F32) {
#pragma unroll
                for (int bx = 0; bx < 4; bx++) tma_load_2d(dst + bx * 8192, map, tc0 + bx * 32, tr0 + k * 64, bar);
            } else {
#pragma unroll
                for (int bx = 0; bx < 8; bx++) tma_load_2d(dst + bx * 4096, map, tc0 + bx * 16, tr0 + k * 32, bar);
            }
            ps.ip = g + 1;
        }
    };

    if (tid == 0) {
        for (int i = 0; i < kStages; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&sm.full[i])) : "memory");
            sm.slot_cnt[i] = 0;
            sm.grp_cnt[i][0] = sm.grp_cnt[i][1] = 0;
        }
        sm.dead = 0;
        ps.n_known = ps.exhausted = ps.stage_end = ps.ip = ps.ip_item = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        claim();
        if (ps.n_known > 0) {
            dep_wait(0);
            claim();
            issue_upto(kStages);
        }
    }
    __syncthreads();

    int lost = -1;
    for (int s = 0; s < ps.n_known; s++) {
        const int e = s & 3;
        const Tile &t = ps.tl[e];
        const int fmt = ps.it[e].fmt, v = ps.it[e].v, group = ps.it[e].group;
        MxInputs &X = sm.sx[s & 1];
        const bool opN = t.k_out0 != VK_NONE, opT = t.k_out1 != VK_NONE;
        /* split the input slices (the dependency was met before the barrier) */
        if (tid < kTileCols) {
            float h = 0.f, l = 0.f;
            if (opN && tid < t.nc) split(__ldcg(vec_ptr(va, t.k_in0, t.in0, v) + tid), h, l);
            X.x0h[tid] = h; X.x0l[tid] = l;
        }
        if (opT) {
            const double *in1 = vec_ptr(va, t.k_in1, t.in1, v);
            for (int r = tid; r < kChunkRows; r += kTileThreads) {   /* rows >= nr read as zero */
                float h = 0.f, l = 0.f;
                if (r < t.nr) split(__ldcg(in1 + r), h, l);
                X.x1h[r] = h; X.x1l[r] = l;
            }
        }
        double *out0 = opN ? vec_ptr(va, t.k_out0, t.out0, v) : nullptr;
        double *out1 = opT ? vec_ptr(va, t.k_out1, t.out1, v) : nullptr;
        __syncthreads();

        const int g0 = ps.gs[e], ns = ps.ns[e];
        float2 ch[2], cl[2];
        ch[0] = ch[1] = cl[0] = cl[1] = make_float2(0.f, 0.f);
        for (int k = 0; k < ns; k++) {
            const int g = g0 + k, slot = g % kStages;
            if (!*dead && !mbar_wait(smem_addr(&sm.full[slot]), (unsigned)((g / kStages) & 1))) {
                atomicOr(err, 1u);
                *dead = 1;
                lost = g;
            }
            if (fmt == FMT_F32) mx_stage<FMT_F32>(sm, slot, t, X, k, k == ns - 1, out0, out1, ch, cl);
            else mx_stage<FMT_F32X2>(sm, slot, t, X, k, k == ns - 1, out0, out1, ch, cl);
            /* release the slot; the last warp out issues the stages it frees */
            if (lane == 0) {
                __threadfence_block();
                if (atomicAdd(&sm.slot_cnt[slot], 1) == NW - 1) {
                    sm.slot_cnt[slot] = 0;
                    __threadfence_block();
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    issue_upto(g + kStages + 1);
                }
            }
        }
        /* the item is done once every thread's output atomics are visible */
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            atomicAdd(&ctl[kPxDone + group], 1);
            if (s + 1 < ps.n_known) {
                dep_wait(s + 1);
                claim();
            }
            issue_upto(g0 + ns + kStages);
        }
        __syncthreads();
    }
    /* copies still in flight after an expired wait: wait for them (bounded) */
    if (tid == 0 && *dead)
        for (int g = max(0, ps.ip - kStages); g < ps.ip; g++)
            (void)mbar_wait(smem_addr(&sm.full[g % kStages]), (unsigned)((g / kStages) & 1));
    if (lost >= 0) (void)mbar_wait(smem_addr(&sm.full[lost % kStages]), (unsigned)((lost / kStages) & 1));
}

/* Self-test of the bounded wait: one CTA waits on an mbarrier (arrival count
 * 1) that nothing arrives at; the wait gives up after `limit` cycles and the
 * error word is set, as in the tile kernels. No copy is in flight, so the CTA
 * exits cleanly. */
__global__ void k_wait_probe(unsigned *err, long long limit)
{
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (!mbar_wait(smem_addr(&bar), 0u, limit) && threadIdx.x == 0) atomicOr(err, 1u);
    __syncthreads();
    if (threadIdx.x == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(&bar)) : "memory");
}

/* x[v][i] = c_i * D[v][map_i >> 1], c_i = 2 for off-diagonal shell pairs
 * (src/H2ERI_build_Coulomb.c:26-62). */
__global__ void k_uncontract(const int *__restrict__ map, int n, const double *__restrict__ den,
                             long long den_stride, double *__restrict__ x, long long x_stride)
{
    const int v = blockIdx.y;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int m = map[i];
        double d = den[v * den_stride + (m >> 1)];
        x[v * x_stride + i] = (m & 1) ? 2.0 * d : d;
    }
}

/* The same as k_uncontract driven by the inverse map (con: D index ->
 * (x index << 1) | diagonal flag, or -1), so the density is read in order:
 * used when it is read in place from host memory, where scattered reads
 * would each cross the host link. Every x entry has exactly one D index. */
__global__ void k_uncontract_scatter(const int *__restrict__ con, long long n2, const double *__restrict__ den,
                                     long long den_stride, double *__restrict__ x, long long x_stride)
{
    const int v = blockIdx.y;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n2; i += (long long)gridDim.x * blockDim.x) {
        const int m = con[i];
        if (m >= 0) {
            const double dv = den[v * den_stride + i];
            x[v * x_stride + (m >> 1)] = (m & 1) ? dv : 2.0 * dv;
        }
    }
}

/* J[a][b] = T[a][b] + T[b][a], T[a][b] = c * y[map >> 1] (c = 0.5 on
 * diagonal shell pairs) or 0 (src/H2ERI_build_Coulomb.c:78-133). */
__global__ void k_contract(const int *__restrict__ map, int nbf, const double *__restrict__ y,
                           long long y_stride, double *__restrict__ J, long long J_stride)
{
    const int v = blockIdx.y;
    const long long n2 = (long long)nbf * nbf;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n2; i += (long long)gridDim.x * blockDim.x) {
        int a = (int)(i / nbf), b = (int)(i - (long long)a * nbf);
        int m1 = map[i], m2 = map[(long long)b * nbf + a];
        double s = 0.0;
        if (m1 >= 0) s += (m1 & 1) ? 0.5 * y[v * y_stride + (m1 >> 1)] : y[v * y_stride + (m1 >> 1)];
        if (m2 >= 0) s += (m2 & 1) ? 0.5 * y[v * y_stride + (m2 >> 1)] : y[v * y_stride + (m2 >> 1)];
        J[v * J_stride + i] = s;
    }
}

/* ======================================================================== */
/* Upload and plan                                                           */
/* ======================================================================== */

static std::mutex g_mu;
static std::unordered_map<const void *, DevRep *> g_reps;

static int noalloc_scratch(int dev, double **out);   /* below, with H2ERI_matvec_device_noalloc */
static void px_free(DevRep *d);                        /* below, with the persistent kernel's work list */

namespace {

/* Location of one stored matrix in the FP64 arena and in the mixed arena of
 * its mixed-mode format. */
struct MatLoc {
    size_t a = 0, a2 = 0;
    int ld = 0, ld2 = 0;
    int map = -1;          /* tensor map of the mixed-arena copy (index of its PackItem) */
    int fmt = FMT_F32;     /* mixed-arena format */
};

/* Packs matrices into the FP64 arena now and records where each goes in the
 * mixed arenas (filled on first use of mixed mode). With trans set the
 * ncol x nrow transpose is stored: tall, narrow matrices (nested bases,
 * low-rank factors, ranks ~50-450) become wide ones that fill 128-column
 * tile strips. Leading dimensions are padded to 16-byte multiples and every
 * matrix starts 32-byte aligned, so rows can be read with 16-byte vector
 * loads; padding is zero. */
struct Packer {
    std::vector<double> host;
    size_t n32 = 0, n32x2 = 0;
    std::vector<PackItem> items;
    MatLoc put(const double *src, int nrow, int ncol, int lds, int mixed_fmt, bool trans = false)
    {
        const int sr = trans ? ncol : nrow, sc = trans ? nrow : ncol;   /* stored shape */
        MatLoc m;
        m.fmt = mixed_fmt;
        m.ld = (sc + 1) & ~1;
        m.a = (host.size() + 3) & ~size_t(3);
        host.resize(m.a + (size_t)sr * m.ld, 0.0);
        for (int r = 0; r < nrow; r++)
            for (int c = 0; c < ncol; c++) {
                const double x = src[(size_t)r * lds + c];
                if (trans) host[m.a + (size_t)c * m.ld + r] = x;
                else host[m.a + (size_t)r * m.ld + c] = x;
            }
        if (mixed_fmt == FMT_F32) {
            m.ld2 = (sc + 3) & ~3;
            m.a2 = (n32 + 7) & ~size_t(7);
            n32 = m.a2 + (size_t)sr * m.ld2;
        } else {
            m.ld2 = (sc + 1) & ~1;
            m.a2 = (n32x2 + 3) & ~size_t(3);
            n32x2 = m.a2 + (size_t)sr * m.ld2;
        }
        m.map = (int)items.size();
        items.push_back(PackItem{src, nrow, ncol, lds, trans ? 1 : 0, mixed_fmt, m.a2, m.ld2});
        return m;
    }
};

/* The tiles of one planned product: chunks of `rows` rows by kTileCols
 * columns. */
void gen_tiles(const PlanRec &q, int rows, std::vector<Tile> &tiles)
{
    for (int r0 = 0; r0 < q.nrow; r0 += rows)
        for (int c0 = 0; c0 < q.ncol; c0 += kTileCols) {
            Tile t;
            std::memset(&t, 0, sizeof(t));
            t.a = q.a + (size_t)r0 * q.ld + c0;
            /* mixed formats: tensor-map coordinates of the tile (TMA loads) */
            t.a2 = ((uint64_t)(uint32_t)c0 << 32) | (uint32_t)r0;
            t.ld = q.ld;
            t.ld2 = q.map;
            t.nr = (int16_t)std::min(rows, q.nrow - r0);
            t.nc = (int16_t)std::min(kTileCols, q.ncol - c0);
            if (q.kout0 != VK_NONE) { t.k_in0 = q.kin0; t.in0 = q.in0 + c0; t.k_out0 = q.kout0; t.out0 = q.out0 + r0; }
            if (q.kout1 != VK_NONE) { t.k_in1 = q.kin1; t.in1 = q.in1 + r0; t.k_out1 = q.kout1; t.out1 = q.out1 + c0; }
            tiles.push_back(t);
        }
}

struct Planner {
    std::vector<Tile> tiles;
    std::vector<TileM> mt;   /* the same products in 128 x 128 tiles (multi-density kernel) */
    std::vector<PlanRec> recs;
    void add(const MatLoc &m, int nrow, int ncol, uint8_t kin0, int in0, uint8_t kout0, int out0,
             uint8_t kin1, int in1, uint8_t kout1, int out1)
    {
        PlanRec q;
        std::memset(&q, 0, sizeof(q));
        q.a = m.a; q.a2 = m.a2; q.ld = m.ld; q.ld2 = m.ld2; q.map = m.map; q.fmt = m.fmt;
        q.nrow = nrow; q.ncol = ncol;
        q.kin0 = kin0; q.in0 = in0; q.kout0 = kout0; q.out0 = out0;
        q.kin1 = kin1; q.in1 = in1; q.kout1 = kout1; q.out1 = out1;
        recs.push_back(q);
        gen_tiles(q, kChunkRows, tiles);
        for (int r0 = 0; r0 < nrow; r0 += kMmaRows)
            for (int c0 = 0; c0 < ncol; c0 += kMmaRows) {
                TileM t;
                std::memset(&t, 0, sizeof(t));
                t.a2 = m.a2 + (size_t)r0 * m.ld2 + c0;
                t.ld2 = m.ld2;
                t.fmt = m.fmt;
                t.nr = (int16_t)std::min(kMmaRows, nrow - r0);
                t.nc = (int16_t)std::min(kMmaRows, ncol - c0);
                if (kout0 != VK_NONE) { t.k_in0 = kin0; t.in0 = in0 + c0; t.k_out0 = kout0; t.out0 = out0 + r0; }
                if (kout1 != VK_NONE) { t.k_in1 = kin1; t.in1 = in1 + r0; t.k_out1 = kout1; t.out1 = out1 + c0; }
                mt.push_back(t);
            }
    }
};

/* A stored B/D block: dense, or low-rank U V with U stored transposed
 * (Ut, rank x nrow) and V stored as is (rank x ncol), both wide. */
struct BlockLoc {
    bool lowrank = false;
    int nrow = 0, ncol = 0, rank = 0;
    MatLoc a, ut, v;
    int t_off = 0, s_off = 0;      /* scratch for t = V in0 and s = U^T in1 */
};

BlockLoc pack_block(Packer &pk, H2E_dense_mat_p m, int &lr_total, int fmt)
{
    BlockLoc b;
    b.nrow = m->nrow;
    b.ncol = m->ncol;
    if (m->ld < 0) {
        b.lowrank = true;
        b.rank = -m->ld;
        b.ut = pk.put(m->data, b.nrow, b.rank, b.rank, fmt, true);
        b.v = pk.put(m->data + (size_t)b.nrow * b.rank, b.ncol, b.rank, b.rank, fmt, true);
        b.t_off = lr_total;
        b.s_off = lr_total + b.rank;
        lr_total += 2 * b.rank;
    } else if ((size_t)b.nrow * b.ncol > 0) {
        b.a = pk.put(m->data, b.nrow, b.ncol, m->ld, fmt);
    }
    return b;
}

/* Stored elements of a block, the reference's block size (nrow ncol, or
 * (nrow + ncol) rank for a low-rank block; src/H2ERI_build_H2.c:869-900):
 * the algorithmic traffic counts every stored element once per matvec. */
double stored_elems(const BlockLoc &b)
{
    if (b.nrow == 0 || b.ncol == 0) return 0.0;
    return b.lowrank ? (double)b.rank * (b.nrow + b.ncol) : (double)b.nrow * b.ncol;
}

/* Products of one block: N-side (out0 += A in0) and T-side (out1 += A^T in1);
 * kinds VK_NONE disable a side. Dense blocks are one bi-product pass. A
 * low-rank block A = U V takes three stages:
 *   1. t = V in0                    (N on V)
 *   2. s = U^T in1, out0 += U t     (one pass over Ut: N and T)
 *   3. out1 += V^T s                (T on V)
 * so U is read once and V twice (each once when only one side is wanted).
 * When U is the smaller factor (nrow < ncol) of a two-sided block, the roles
 * swap and U is the one read twice:
 *   1. s = U^T in1                  (N on Ut)
 *   2. t = V in0, out1 += V^T s     (one pass over V: N and T)
 *   3. out0 += U t                  (T on Ut) */
void plan_block(Planner *st, const BlockLoc &b, uint8_t kin0, int in0, uint8_t kout0, int out0, uint8_t kin1,
                int in1, uint8_t kout1, int out1)
{
    if (b.nrow == 0 || b.ncol == 0) return;
    if (!b.lowrank) {
        st[0].add(b.a, b.nrow, b.ncol, kin0, in0, kout0, out0, kin1, in1, kout1, out1);
        return;
    }
    const int r = b.rank;
    if (r == 0) return;
    const bool wantN = kout0 != VK_NONE, wantT = kout1 != VK_NONE;
    if (wantN && wantT && b.nrow < b.ncol) {
        st[0].add(b.ut, r, b.nrow, kin1, in1, VK_T, b.s_off, VK_NONE, 0, VK_NONE, 0);
        st[1].add(b.v, r, b.ncol, kin0, in0, VK_T, b.t_off, VK_T, b.s_off, kout1, out1);
        st[2].add(b.ut, r, b.nrow, VK_NONE, 0, VK_NONE, 0, VK_T, b.t_off, kout0, out0);
        return;
    }
    if (wantN) st[0].add(b.v, r, b.ncol, kin0, in0, VK_T, b.t_off, VK_NONE, 0, VK_NONE, 0);
    st[1].add(b.ut, r, b.nrow, wantT ? kin1 : VK_NONE, in1, wantT ? VK_T : VK_NONE, b.s_off,
              wantN ? VK_T : VK_NONE, b.t_off, wantN ? kout0 : VK_NONE, out0);
    if (wantT) st[2].add(b.v, r, b.ncol, VK_NONE, 0, VK_NONE, 0, VK_T, b.s_off, kout1, out1);
}

}  // namespace

static void free_rep(DevRep *d)
{
    if (d == nullptr) return;
    int cur = -1;
    cudaGetDevice(&cur);
    if (d->device >= 0) cudaSetDevice(d->device);
    cudaFree(d->arena);
    cudaFree(d->arena32);
    cudaFree(d->arena32x2);
    cudaFree(d->tmaps);
    if (d->err_flag) cudaFreeHost(d->err_flag);
    cudaFree(d->tiles);
    cudaFree(d->mtiles);
    cudaFree(d->mscales);
    cudaFree(d->mslices);
    cudaFree(d->unc_map);
    cudaFree(d->con_map);
    cudaFree(d->work);
    cudaFree(d->xbuf);
    cudaFree(d->ybuf);
    cudaFree(d->dbuf);
    cudaFree(d->jbuf);
    if (d->s_main) cudaStreamDestroy(d->s_main);
    if (d->s_aux) cudaStreamDestroy(d->s_aux);
    for (int i = 1; i < kNfLanes; i++) {
        if (d->s_nf[i]) cudaStreamDestroy(d->s_nf[i]);
        if (d->ev_nf[i]) cudaEventDestroy(d->ev_nf[i]);
    }
    if (d->ev_fork) cudaEventDestroy(d->ev_fork);
    if (d->ev_join) cudaEventDestroy(d->ev_join);
    if (d->ev_zero) cudaEventDestroy(d->ev_zero);
    if (d->ev_done) cudaEventDestroy(d->ev_done);
    if (d->ev_bfork) cudaEventDestroy(d->ev_bfork);
    if (d->ev_bjoin) cudaEventDestroy(d->ev_bjoin);
    for (auto &e : d->ev_t)
        if (e) cudaEventDestroy(e);
    px_free(d);
    free_exchange_state(d);
    batch_forget(d);
    if (cur >= 0) cudaSetDevice(cur);
    delete d;
}

/* Host-side bounds check of the launch plan before anything reaches the
 * device: every vector range a tile reads or adds to lies inside its vector,
 * every tile lies inside the FP64 arena, and the tile shapes fit the
 * kernels. A structure with damaged tree arrays (a corrupted file, a
 * caller's mistake) is rejected here instead of faulting a kernel. */
static bool plan_in_bounds(const std::vector<Tile> &tiles, size_t arena_elems, long long krnl, long long rank_total,
                           long long lr_total, std::string &why)
{
    auto len = [&](uint8_t k) -> long long {
        switch (k) {
        case VK_X: case VK_Y: return krnl;
        case VK_Y0: case VK_Y1: return rank_total;
        case VK_T: return lr_total;
        default: return -1;
        }
    };
    auto range_ok = [&](uint8_t k, long long off, long long n) {
        const long long L = len(k);
        return L >= 0 && off >= 0 && off + n <= L;
    };
    for (size_t i = 0; i < tiles.size(); i++) {
        const Tile &t = tiles[i];
        const bool n_side = t.k_out0 != VK_NONE, t_side = t.k_out1 != VK_NONE;
        bool ok = (n_side || t_side) && t.nr >= 1 && t.nr <= kChunkRows && t.nc >= 1 && t.nc <= kTileCols &&
                  t.ld >= t.nc && t.a + (uint64_t)(t.nr - 1) * (uint64_t)t.ld + (uint64_t)((t.nc + 1) & ~1) <= arena_elems;
        if (ok && n_side) ok = range_ok(t.k_in0, t.in0, t.nc) && range_ok(t.k_out0, t.out0, t.nr);
        if (ok && t_side) ok = range_ok(t.k_in1, t.in1, t.nr) && range_ok(t.k_out1, t.out1, t.nc);
        if (!ok) {
            why = "launch plan out of bounds at tile " + std::to_string(i) + " (damaged tree arrays or blocks)";
            return false;
        }
    }
    return true;
}

static int build_rep(H2ERI_p h, DevRep *d)
{
    if (h->U == nullptr || h->c_D_blks == nullptr || (h->n_B > 0 && h->c_B_blks == nullptr)) {
        set_error("H2 representation not built (call H2ERI_build_H2 with BD_JIT = 0)");
        return 2;
    }
    const int n_node = h->n_node, krnl = h->krnl_mat_size;
    Packer pk;
    pk.host.reserve((size_t)(h->mat_size[U_SIZE_IDX] + h->mat_size[B_SIZE_IDX] + h->mat_size[D_SIZE_IDX]) + 4096);

    /* coefficient segments: children of a node are contiguous, in child order */
    std::vector<int> voff(n_node, -1), rank(n_node, 0);
    for (int i = 0; i < n_node; i++) rank[i] = h->U[i]->ncol;
    int rtot = 0;
    voff[h->root_idx] = rtot;
    rtot += rank[h->root_idx];
    for (int lv = 0; lv <= h->max_level; lv++)
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = h->level_nodes[lv * h->n_leaf_node + j];
            for (int k = 0; k < h->n_child[node]; k++) {
                int c = h->children[node * h->max_child + k];
                voff[c] = rtot;
                rtot += rank[c];
            }
        }
    d->rank_total = rtot;

    /* which upward / downward coefficients are ever non-zero */
    std::vector<char> used_y0(n_node, 0), wrote_y1(n_node, 0);
    for (int i = 0; i < h->n_r_adm_pair; i++) {
        int n0 = h->r_adm_pairs[2 * i], n1 = h->r_adm_pairs[2 * i + 1];
        int l0 = h->node_level[n0], l1 = h->node_level[n1];
        if (l0 >= l1) { used_y0[n0] = 1; wrote_y1[n0] = 1; }
        if (l0 <= l1) { used_y0[n1] = 1; wrote_y1[n1] = 1; }
    }
    std::vector<char> need_up(n_node, 0), need_down(n_node, 0);
    for (int lv = h->min_adm_level; lv <= h->max_level; lv++)
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = h->level_nodes[lv * h->n_leaf_node + j];
            int p = h->parent[node];
            bool pin = p >= 0 && h->node_level[p] >= h->min_adm_level;
            need_up[node] = used_y0[node] || (pin && need_up[p]);
            need_down[node] = wrote_y1[node] || (pin && need_down[p] && rank[p] > 0);
        }

    Planner midst[3], dend[3], deno[kNfLanes][3];
    double lane_load[kNfLanes] = {0.0};
    std::vector<Tile> all;
    std::vector<TileM> mall;
    d->mfwd.clear();
    d->mbwd.clear();
    d->mmid.clear();
    d->mden.clear();
    d->rec_fwd.clear();
    d->rec_mid.clear();
    d->rec_bwd.clear();
    d->rec_den.clear();
    double mat_bytes = 0.0, mat_bytes_mixed = 0.0, vec_bytes = 0.0, flops = 0.0;
    d->fwd.clear();
    d->bwd.clear();

    /* U bases */
    std::vector<MatLoc> uloc(n_node);
    for (int i = 0; i < n_node; i++) {
        H2E_dense_mat_p U = h->U[i];
        /* stored transposed (rank x rows): wide, fills the 128-column strips */
        if (U->nrow > 0 && U->ncol > 0) uloc[i] = pk.put(U->data, U->nrow, U->ncol, U->ld, FMT_F32X2, true);
    }
    d->bytes_U = pk.host.size() * sizeof(double);

    /* upward sweep, deepest level first (src/H2ERI_matvec.c:111-156) */
    for (int lv = h->max_level; lv >= h->min_adm_level; lv--) {
        Planner p;
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = h->level_nodes[lv * h->n_leaf_node + j];
            H2E_dense_mat_p U = h->U[node];
            if (!need_up[node] || U->nrow == 0 || U->ncol == 0) continue;
            bool leaf = h->n_child[node] == 0;
            int in_off = leaf ? h->mat_cluster[2 * node] : voff[h->children[node * h->max_child]];
            /* y0 = U^T in = Ut in: N side of the stored transpose */
            p.add(uloc[node], U->ncol, U->nrow, leaf ? VK_X : VK_Y0, in_off, VK_Y0, voff[node], VK_NONE, 0,
                  VK_NONE, 0);
            mat_bytes += 8.0 * U->nrow * U->ncol;
            mat_bytes_mixed += 8.0 * U->nrow * U->ncol;
            vec_bytes += 8.0 * (U->nrow + U->ncol);
            flops += 2.0 * U->nrow * U->ncol;
        }
        Range r{(int)all.size(), (int)p.tiles.size(), true};
        all.insert(all.end(), p.tiles.begin(), p.tiles.end());
        d->fwd.push_back(r);
        d->mfwd.push_back(Range{(int)mall.size(), (int)p.mt.size(), true});
        mall.insert(mall.end(), p.mt.begin(), p.mt.end());
        d->rec_fwd.push_back(std::move(p.recs));
    }

    /* coupling blocks (src/H2ERI_matvec.c:299-407) */
    size_t b_start = pk.host.size();
    for (int i = 0; i < h->n_r_adm_pair; i++) {
        int n0 = h->r_adm_pairs[2 * i], n1 = h->r_adm_pairs[2 * i + 1];
        int l0 = h->node_level[n0], l1 = h->node_level[n1];
        BlockLoc b = pack_block(pk, h->c_B_blks[i], d->lr_total, FMT_F32);
        uint8_t kin0, kout0, kin1, kout1;
        int in0, out0, in1, out1;
        if (l0 == l1) {
            kin0 = VK_Y0; in0 = voff[n1]; kout0 = VK_Y1; out0 = voff[n0];
            kin1 = VK_Y0; in1 = voff[n0]; kout1 = VK_Y1; out1 = voff[n1];
        } else if (l0 > l1) {
            kin0 = VK_X; in0 = h->mat_cluster[2 * n1]; kout0 = VK_Y1; out0 = voff[n0];
            kin1 = VK_Y0; in1 = voff[n0]; kout1 = VK_Y; out1 = h->mat_cluster[2 * n1];
        } else {
            kin0 = VK_Y0; in0 = voff[n1]; kout0 = VK_Y; out0 = h->mat_cluster[2 * n0];
            kin1 = VK_X; in1 = h->mat_cluster[2 * n0]; kout1 = VK_Y1; out1 = voff[n1];
        }
        plan_block(midst, b, kin0, in0, kout0, out0, kin1, in1, kout1, out1);
        const double el = stored_elems(b);
        mat_bytes += 8.0 * el;
        mat_bytes_mixed += 4.0 * el;
        vec_bytes += 8.0 * 2 * (b.nrow + b.ncol);
        flops += 4.0 * el;
    }
    d->bytes_B = (pk.host.size() - b_start) * sizeof(double);
    d->mid.clear();
    for (int k = 0; k < 3; k++) {
        d->mid.push_back(Range{(int)all.size(), (int)midst[k].tiles.size(), false});
        all.insert(all.end(), midst[k].tiles.begin(), midst[k].tiles.end());
        d->mmid.push_back(Range{(int)mall.size(), (int)midst[k].mt.size(), false});
        mall.insert(mall.end(), midst[k].mt.begin(), midst[k].mt.end());
        d->rec_mid.push_back(std::move(midst[k].recs));
    }

    /* downward sweep, shallowest level first (src/H2ERI_matvec.c:679-738) */
    for (int lv = h->min_adm_level; lv <= h->max_level; lv++) {
        Planner p;
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = h->level_nodes[lv * h->n_leaf_node + j];
            H2E_dense_mat_p U = h->U[node];
            if (!need_down[node] || U->nrow == 0 || U->ncol == 0) continue;
            bool leaf = h->n_child[node] == 0;
            int out_off = leaf ? h->mat_cluster[2 * node] : voff[h->children[node * h->max_child]];
            /* out += U y1 = Ut^T y1: T side of the stored transpose */
            p.add(uloc[node], U->ncol, U->nrow, VK_NONE, 0, VK_NONE, 0, VK_Y1, voff[node], leaf ? VK_Y : VK_Y1,
                  out_off);
            mat_bytes += 8.0 * U->nrow * U->ncol;
            mat_bytes_mixed += 8.0 * U->nrow * U->ncol;
            vec_bytes += 8.0 * (U->nrow + U->ncol);
            flops += 2.0 * U->nrow * U->ncol;
        }
        Range r{(int)all.size(), (int)p.tiles.size(), true};
        all.insert(all.end(), p.tiles.begin(), p.tiles.end());
        d->bwd.push_back(r);
        d->mbwd.push_back(Range{(int)mall.size(), (int)p.mt.size(), true});
        mall.insert(mall.end(), p.mt.begin(), p.mt.end());
        d->rec_bwd.push_back(std::move(p.recs));
    }

    /* near field (src/H2ERI_matvec.c:572-660) */
    size_t d_start = pk.host.size();
    for (int i = 0; i < h->n_D; i++) {
        /* mixed mode keeps the leaf self-interaction blocks as float pairs */
        const bool diag = i < h->n_leaf_node;
        BlockLoc b = pack_block(pk, h->c_D_blks[i], d->lr_total, diag ? FMT_F32X2 : FMT_F32);
        const double el = stored_elems(b);
        if (diag) {
            int node = h->height_nodes[i];
            int off = h->mat_cluster[2 * node];
            plan_block(dend, b, VK_X, off, VK_Y, off, VK_NONE, 0, VK_NONE, 0);
            vec_bytes += 8.0 * (b.nrow + b.ncol);
            flops += 2.0 * el;
        } else {
            int k = i - h->n_leaf_node;
            int n0 = h->r_inadm_pairs[2 * k], n1 = h->r_inadm_pairs[2 * k + 1];
            int o0 = h->mat_cluster[2 * n0], o1 = h->mat_cluster[2 * n1];
            /* single-float blocks: the least-loaded lane (stored elements) */
            int ln = 1;
            for (int q = 2; q < kNfLanes; q++)
                if (lane_load[q] < lane_load[ln]) ln = q;
            lane_load[ln] += el;
            plan_block(deno[ln], b, VK_X, o1, VK_Y, o0, VK_X, o0, VK_Y, o1);
            vec_bytes += 8.0 * 2 * (b.nrow + b.ncol);
            flops += 4.0 * el;
        }
        mat_bytes += 8.0 * el;
        mat_bytes_mixed += (diag ? 8.0 : 4.0) * el;
    }
    d->bytes_D = (pk.host.size() - d_start) * sizeof(double);
    /* near-field lanes: lane 0 the float-pair blocks, lanes 1.. groups of
     * single-float blocks; each lane's three stages form an independent
     * chain on its own stream */
    d->den.clear();
    for (int ln = 0; ln < kNfLanes; ln++)
        for (int k = 0; k < 3; k++) {
            Planner &p = ln == 0 ? dend[k] : deno[ln][k];
            d->den.push_back(Range{(int)all.size(), (int)p.tiles.size(), ln == 0, ln});
            all.insert(all.end(), p.tiles.begin(), p.tiles.end());
            d->mden.push_back(Range{(int)mall.size(), (int)p.mt.size(), ln == 0, ln});
            mall.insert(mall.end(), p.mt.begin(), p.mt.end());
            d->rec_den.push_back(std::move(p.recs));
        }

    d->alg_bytes_matrix = mat_bytes;
    d->alg_bytes_matrix_mixed = mat_bytes_mixed;
    d->mixed_items = std::move(pk.items);
    d->arena32_elems = pk.n32;
    d->arena32x2_elems = pk.n32x2;
    d->alg_bytes_vec = vec_bytes;
    d->alg_flops = flops;
    d->n_tiles = (int)all.size();
    d->arena_elems = pk.host.size();
    {
        std::string why;
        if (!plan_in_bounds(all, d->arena_elems, krnl, d->rank_total, d->lr_total, why)) {
            set_error(why);
            return 3;
        }
    }
    CUDA_TRY(cudaMalloc(&d->arena, std::max<size_t>(d->arena_elems, 4) * sizeof(double)));
    CUDA_TRY(cudaMemcpy(d->arena, pk.host.data(), d->arena_elems * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMalloc(&d->tiles, std::max<size_t>(all.size(), 1) * sizeof(Tile)));
    if (!all.empty()) CUDA_TRY(cudaMemcpy(d->tiles, all.data(), all.size() * sizeof(Tile), cudaMemcpyHostToDevice));
    d->tiles_host = all;
    d->n_mtiles = (int)mall.size();
    {
        /* offsets of the tiles' pre-computed slices (1 KB aligned) */
        size_t off = 0;
        for (TileM &t : mall) {
            t.s_off = off;
            off += (size_t)4 * ((t.nc + 63) / 64) * ((t.nr + 7) / 8) * 1024;
        }
        d->mslice_bytes = off;
    }
    CUDA_TRY(cudaMalloc(&d->mtiles, std::max<size_t>(mall.size(), 1) * sizeof(TileM)));
    if (!mall.empty()) CUDA_TRY(cudaMemcpy(d->mtiles, mall.data(), mall.size() * sizeof(TileM), cudaMemcpyHostToDevice));
    d->mtiles_host = std::move(mall);

    /* J assembly maps */
    const int nbf = h->num_bf, num_sp = h->num_sp;
    std::vector<int> unc(std::max(krnl, 1), 0), con((size_t)nbf * nbf, -1);
    for (int i = 0; i < num_sp; i++) {
        int M = h->sp_shell_idx[i], N = h->sp_shell_idx[i + num_sp];
        int srow = h->shell_bf_sidx[M], nrow = h->shell_bf_sidx[M + 1] - srow;
        int scol = h->shell_bf_sidx[N], ncol = h->shell_bf_sidx[N + 1] - scol;
        int base = h->sp_bfp_sidx[i];
        for (int j = 0; j < ncol; j++)
            for (int k = 0; k < nrow; k++) {
                int xi = base + j * nrow + k;
                int di = (scol + j) * nbf + srow + k;
                if (xi < 0 || xi >= krnl || di < 0 || (long long)di >= (long long)nbf * nbf) {
                    set_error("J maps out of bounds (damaged shell-pair arrays)");
                    return 3;
                }
                unc[xi] = (di << 1) | (M != N ? 1 : 0);
                con[di] = (xi << 1) | (M == N ? 1 : 0);
            }
    }
    CUDA_TRY(cudaMalloc(&d->unc_map, unc.size() * sizeof(int)));
    CUDA_TRY(cudaMemcpy(d->unc_map, unc.data(), unc.size() * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMalloc(&d->con_map, std::max<size_t>(con.size(), 1) * sizeof(int)));
    CUDA_TRY(cudaMemcpy(d->con_map, con.data(), con.size() * sizeof(int), cudaMemcpyHostToDevice));

    CUDA_TRY(cudaHostAlloc((void **)&d->err_flag, sizeof(unsigned), cudaHostAllocMapped));
    *d->err_flag = 0;
    CUDA_TRY(cudaHostGetDevicePointer((void **)&d->err_flag_dev, d->err_flag, 0));
    CUDA_TRY(cudaFuncSetAttribute(k_tile<FMT_F64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmemLaunch));
    CUDA_TRY(cudaFuncSetAttribute(k_tile_mx<FMT_F32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMxSmem));
    CUDA_TRY(cudaFuncSetAttribute(k_tile_mx<FMT_F32X2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMxSmem));
    CUDA_TRY(cudaFuncSetAttribute(k_tile_mx<FMT_F32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMxSmem));
    CUDA_TRY(cudaFuncSetAttribute(k_tile_mx<FMT_F32X2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMxSmem));
    CUDA_TRY(cudaFuncSetAttribute(k_tile_px, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPxSmem));
    {
        int rc = mma_init(d);
        if (rc) return rc;
    }
    /* The tree sweeps are a chain of dependent launches (the critical path);
     * the near field is one large independent batch. Giving the chain's
     * stream the higher priority lets near-field tiles fill only the SMs the
     * chain leaves idle. */
    int prio_lo = 0, prio_hi = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
    CUDA_TRY(cudaStreamCreateWithPriority(&d->s_main, cudaStreamNonBlocking, prio_hi));
    CUDA_TRY(cudaStreamCreateWithPriority(&d->s_aux, cudaStreamNonBlocking, prio_lo));
    for (int i = 1; i < kNfLanes; i++) {
        CUDA_TRY(cudaStreamCreateWithPriority(&d->s_nf[i], cudaStreamNonBlocking, prio_lo));
        CUDA_TRY(cudaEventCreateWithFlags(&d->ev_nf[i], cudaEventDisableTiming));
    }
    CUDA_TRY(cudaEventCreateWithFlags(&d->ev_fork, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&d->ev_join, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&d->ev_zero, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&d->ev_done, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&d->ev_bfork, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&d->ev_bjoin, cudaEventDisableTiming));
    for (auto &e : d->ev_t) CUDA_TRY(cudaEventCreate(&e));

    /* the address of the fixed scratch array of H2ERI_matvec_device_noalloc
     * on this device, resolved here so that the allocation-free call itself
     * only reads it (the lookup may load this module's device code) */
    {
        int rc = noalloc_scratch(d->device, &d->noalloc_work);
        if (rc) return rc;
    }

    d->krnl = krnl;
    d->n_node = n_node;
    d->num_bf = nbf;
    d->n_B = h->n_B;
    d->n_D = h->n_D;
    d->fp_U = h->U;
    d->fp_B = h->c_B_blks;
    d->fp_D = h->c_D_blks;
    return 0;
}

/* Rebuild the single-density tile plan with tiles of `rows` rows (a
 * multiple of 64, at most kChunkRows), from the recorded products: same
 * ranges, same arenas. Waits for the device first (the old tile list may be
 * in use). */
/* Rows per tile of one range in the adaptive plan: the tallest of 512, 256,
 * 128, 64 that still gives the range at least two waves of CTAs (two tiles
 * per CTA, two CTAs per SM). A range with few, tall tiles (the narrow levels
 * of the tree) is otherwise bound by a few CTAs streaming long tiles one
 * stage at a time, while wide ranges keep tall tiles and their lower
 * per-CTA overhead. */
static int adaptive_rows(const std::vector<PlanRec> &recs, int n_sm)
{
    const long long want = 2LL * 2 * 2 * std::max(n_sm, 1);   /* tiles for two waves */
    int rows = kChunkRows;
    for (; rows > 64; rows /= 2) {
        long long n = 0;
        for (const PlanRec &q : recs)
            n += (long long)((q.nrow + rows - 1) / rows) * ((q.ncol + kTileCols - 1) / kTileCols);
        if (n >= want) break;
    }
    return rows;
}

/* Rebuild the tile plan from the recorded products with `rows` rows per tile
 * (a multiple of 64 up to 512), or per range with adaptive_rows (rows 0). */
int replan_tiles(DevRep *d, int rows)
{
    if (rows != 0 && (rows < 64 || rows > kChunkRows || rows % 64 != 0)) {
        set_error("tile rows must be 0 (per range) or a multiple of 64 in [64, " + std::to_string(kChunkRows) + "]");
        return 3;
    }
    if (rows == d->cfg.chunk_rows && d->tiles != nullptr) return 0;
    std::vector<Tile> all;
    auto emit = [&](std::vector<Range> &rr, const std::vector<std::vector<PlanRec>> &recs) {
        for (size_t k = 0; k < rr.size() && k < recs.size(); k++) {
            rr[k].first = (int)all.size();
            const int rk = rows ? rows : adaptive_rows(recs[k], d->n_sm);
            for (const PlanRec &q : recs[k]) gen_tiles(q, rk, all);
            rr[k].count = (int)all.size() - rr[k].first;
        }
    };
    emit(d->fwd, d->rec_fwd);
    emit(d->mid, d->rec_mid);
    emit(d->bwd, d->rec_bwd);
    emit(d->den, d->rec_den);
    std::string why;
    if (!plan_in_bounds(all, d->arena_elems, d->krnl, d->rank_total, d->lr_total, why)) {
        set_error(why);
        return 3;
    }
    CUDA_TRY(cudaDeviceSynchronize());
    Tile *nt = nullptr;
    CUDA_TRY(cudaMalloc(&nt, std::max<size_t>(all.size(), 1) * sizeof(Tile)));
    if (!all.empty()) CUDA_TRY(cudaMemcpy(nt, all.data(), all.size() * sizeof(Tile), cudaMemcpyHostToDevice));
    cudaFree(d->tiles);
    d->tiles = nt;
    d->n_tiles = (int)all.size();
    d->tiles_host = std::move(all);
    px_free(d);   /* the persistent kernel's work list names tiles of the old plan */
    d->cfg.chunk_rows = rows;
    return 0;
}

/* Launch choices fixed through the environment; they take precedence over
 * the defaults and over choices tuned earlier (applied after those):
 *   H2G_MMA_LEVELS=4|5      slice levels of the multi-density kernel
 *   H2G_MMA_MIN_VEC=n       densities per launch from which it runs
 *   H2G_TILE_ROWS=128|256|512, H2G_TILES_PER_CTA=1|2
 *   H2G_PERSIST=0|1         mixed single-density matvec as one persistent launch */
static int apply_env_choices(DevRep *d)
{
    if (const char *lv = std::getenv("H2G_MMA_LEVELS")) d->mma_levels = std::atoi(lv) == 4 ? 4 : 5;
    if (const char *mv = std::getenv("H2G_MMA_MIN_VEC")) d->cfg.mma_min_vec = std::max(2, std::atoi(mv));
    if (const char *tr = std::getenv("H2G_TILE_ROWS")) {
        const int rc = replan_tiles(d, std::atoi(tr));
        if (rc) return rc;
    }
    if (const char *tp = std::getenv("H2G_TILES_PER_CTA")) d->cfg.tiles_per_cta = std::atoi(tp) == 1 ? 1 : 2;
    if (const char *pp = std::getenv("H2G_PERSIST")) d->cfg.persist = std::atoi(pp) == 0 ? 0 : 1;
    return 0;
}

/* Look up (and if needed create) the device representation of h. */
int get_rep(H2ERI_p h, DevRep **out)
{
    if (h == nullptr) { set_error("null H2ERI handle"); return 1; }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        set_error(std::string("no usable CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices"));
        return 9;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_reps.find(h);
    if (it != g_reps.end()) {
        DevRep *d = it->second;
        if (d->krnl == h->krnl_mat_size && d->n_node == h->n_node && d->fp_U == h->U && d->fp_B == h->c_B_blks &&
            d->fp_D == h->c_D_blks) {
            *out = d;
            return 0;
        }
        free_rep(d);         /* stale: the structure was rebuilt */
        g_reps.erase(it);
    }
    DevRep *d = new DevRep();
    cudaGetDevice(&d->device);
    int rc = build_rep(h, d);
    if (rc != 0) { free_rep(d); return rc; }
    tune_apply_cached(d);   /* launch choices tuned earlier for this shape (H2G_TUNE_FILE) */
    rc = apply_env_choices(d);
    if (rc) { free_rep(d); return rc; }
    /* H2G_PRECISION=mixed starts the structure in the mixed mode, for callers
     * of the reference's entry points that do not call the extensions */
    if (const char *pe = std::getenv("H2G_PRECISION")) {
        if (std::strcmp(pe, "mixed") == 0) {
            rc = set_precision_mode(d, h, H2ERI_GPU_MIXED);
            if (rc != 0) { free_rep(d); return rc; }
        } else if (pe[0] != '\0' && std::strcmp(pe, "fp64") != 0) {
            set_error(std::string("H2G_PRECISION must be fp64 or mixed, not ") + pe);
            free_rep(d);
            return 3;
        }
    }
    g_reps[h] = d;
    *out = d;
    return 0;
}

int ensure_work(DevRep *d, int nvec)
{
    if (nvec <= d->nvec_cap) return 0;
    cudaFree(d->work);
    cudaFree(d->xbuf);
    cudaFree(d->ybuf);
    d->work = d->xbuf = d->ybuf = nullptr;
    size_t per = (size_t)2 * d->rank_total + d->lr_total;
    CUDA_TRY(cudaMalloc(&d->work, std::max<size_t>(per * nvec, 1) * sizeof(double)));
    CUDA_TRY(cudaMalloc(&d->xbuf, (size_t)std::max(d->krnl, 1) * nvec * sizeof(double)));
    CUDA_TRY(cudaMalloc(&d->ybuf, (size_t)std::max(d->krnl, 1) * nvec * sizeof(double)));
    d->nvec_cap = nvec;
    return 0;
}

/* Mixed mode picks the float-pair kernel for ranges marked pair (U bases,
 * near-field diagonal blocks) and the single-float kernel otherwise. */
static void launch_range(const DevRep *d, const Range &r, const VecArgs &va, int nvec, cudaStream_t s)
{
    constexpr int kMaxGridY = 65535;
    for (int f = 0; f < r.count; f += kMaxGridY) {
        dim3 grid(nvec, std::min(kMaxGridY, r.count - f));
        const Tile *t = d->tiles + r.first + f;
        const CUtensorMap *maps = reinterpret_cast<const CUtensorMap *>(d->tmaps);
        if (d->precision == H2ERI_GPU_FP64)
            k_tile<FMT_F64><<<grid, kTileThreads, kTileSmemLaunch, s>>>(t, d->arena, va);
        else {
            /* two tiles per CTA: tiles y and y + half of this launch (one
             * per CTA when the grid covers every tile) */
            const int n = std::min(kMaxGridY, r.count - f);
            dim3 g2(nvec, d->cfg.tiles_per_cta == 1 ? n : (n + 1) / 2);
            if (r.pair)
                k_tile_mx<FMT_F32X2, false><<<g2, kTileThreads, kMxSmem, s>>>(t, n, va, maps, d->err_flag_dev, nullptr);
            else
                k_tile_mx<FMT_F32, false><<<g2, kTileThreads, kMxSmem, s>>>(t, n, va, maps, d->err_flag_dev, nullptr);
        }
    }
}

/* One merged range of a batch plan on the mixed single-density kernel:
 * tiles of every structure (structure index in Tile::a), the structures'
 * tensor maps concatenated, nvec densities each. */
void launch_batch_mx(const Tile *tiles, int count, bool pair, const void *maps, const BatchMol *mols, int nvec,
                     int tiles_per_cta, unsigned *err, cudaStream_t s)
{
    constexpr int kMaxGridY = 65535;
    VecArgs none;
    std::memset(&none, 0, sizeof(none));
    for (int f = 0; f < count; f += kMaxGridY) {
        const int n = std::min(kMaxGridY, count - f);
        dim3 g2(nvec, tiles_per_cta == 1 ? n : (n + 1) / 2);
        const CUtensorMap *m = reinterpret_cast<const CUtensorMap *>(maps);
        if (pair)
            k_tile_mx<FMT_F32X2, true><<<g2, kTileThreads, kMxSmem, s>>>(tiles + f, n, none, m, err, mols);
        else
            k_tile_mx<FMT_F32, true><<<g2, kTileThreads, kMxSmem, s>>>(tiles + f, n, none, m, err, mols);
    }
}

/* cuTensorMapEncodeTiled, looked up through the runtime (no link-time
 * dependency on the driver library). */
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

/* One tensor map per matrix of the mixed arenas: a 2-D view (leading
 * dimension as the extent, so the zero padding of a row is in range; float
 * pairs as 8-byte elements) with boxes of 128 bytes x one stage of rows and
 * the 128-byte swizzle; rows and columns outside the matrix read as zero. */
static int build_tensor_maps(DevRep *d)
{
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (fn == nullptr || q != cudaDriverEntryPointSuccess) {
        set_error("cuTensorMapEncodeTiled is not available");
        return 10;
    }
    const EncodeTiledFn encode = reinterpret_cast<EncodeTiledFn>(fn);
    std::vector<CUtensorMap> maps(std::max<size_t>(d->mixed_items.size(), 1));
    for (size_t i = 0; i < d->mixed_items.size(); i++) {
        const PackItem &it = d->mixed_items[i];
        const bool pair = it.fmt == FMT_F32X2;
        const int eb = pair ? 8 : 4;
        const int srows = it.trans ? it.ncol : it.nrow;
        unsigned char *base = pair ? reinterpret_cast<unsigned char *>(d->arena32x2) + it.off * 8
                                   : reinterpret_cast<unsigned char *>(d->arena32) + it.off * 4;
        const cuuint64_t dims[2] = {(cuuint64_t)it.ld, (cuuint64_t)std::max(srows, 1)};
        const cuuint64_t strides[1] = {(cuuint64_t)it.ld * eb};
        const cuuint32_t box[2] = {(cuuint32_t)(kTmaBoxBytes / eb), (cuuint32_t)(kStageBytes / (kTileCols * eb))};
        const cuuint32_t estr[2] = {1, 1};
        const CUresult r = encode(&maps[i], pair ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                  base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
            set_error("cuTensorMapEncodeTiled failed for mixed matrix " + std::to_string(i) + " (code " +
                      std::to_string((int)r) + ")");
            return 10;
        }
    }
    CUDA_TRY(cudaMalloc(&d->tmaps, maps.size() * sizeof(CUtensorMap)));
    CUDA_TRY(cudaMemcpy(d->tmaps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
    return 0;
}

/* Power-of-two equilibration of every multi-density tile (from the values
 * as stored in the mixed arenas): row exponents e_r with max_c |A_rc| <
 * 2^e_r, then column exponents f_c with max_r |A_rc| 2^-e_r < 2^f_c, so the
 * scaled tile A_rc 2^-(e_r + f_c) lies in (-1, 1); 128 row then 128 column
 * int8 values per tile, clamped to [-126, 126] (zero rows and columns get
 * 0). Each tile is also checked against its arena before upload. */
static int mma_scales(DevRep *d, const std::vector<float> &h32, const std::vector<float2> &h32x2)
{
    const int n = d->n_mtiles;
    std::vector<int8_t> sc((size_t)std::max(n, 1) * 256, 0);
    const float *f2 = reinterpret_cast<const float *>(h32x2.data());
    bool bad = false;
#pragma omp parallel for schedule(dynamic, 16) reduction(|| : bad)
    for (int t = 0; t < n; t++) {
        const TileM &T = d->mtiles_host[t];
        const bool pair = T.fmt == FMT_F32X2;
        const size_t lim = pair ? h32x2.size() : h32.size();
        if (T.nr < 1 || T.nr > kMmaRows || T.nc < 1 || T.nc > kMmaRows || T.ld2 < T.nc ||
            T.a2 + (size_t)(T.nr - 1) * T.ld2 + (size_t)T.nc > lim) {
            bad = true;
            continue;
        }
        auto val = [&](int r, int c) -> double {
            const size_t pos = T.a2 + (size_t)r * T.ld2 + c;
            if (!pair) return (double)h32[pos];
            const size_t e = pos & ~size_t(1), k = pos & 1;
            return (double)f2[2 * e + k] + (double)f2[2 * e + 2 + k];
        };
        auto expo = [](double m) -> int {
            if (!(m > 0.0)) return 0;
            int ex;
            std::frexp(m, &ex);   /* m < 2^ex */
            return std::min(126, std::max(-126, ex));
        };
        int8_t *out = sc.data() + (size_t)t * 256;
        int er[kMmaRows] = {0};
        for (int r = 0; r < T.nr; r++) {
            double m = 0.0;
            for (int c = 0; c < T.nc; c++) m = std::max(m, std::fabs(val(r, c)));
            er[r] = expo(m);
            out[r] = (int8_t)er[r];
        }
        for (int c = 0; c < T.nc; c++) {
            double m = 0.0;
            for (int r = 0; r < T.nr; r++) m = std::max(m, std::ldexp(std::fabs(val(r, c)), -er[r]));
            out[128 + c] = (int8_t)expo(m);
        }
    }
    if (bad) {
        set_error("multi-density tile outside its mixed arena (damaged plan)");
        return 3;
    }
    CUDA_TRY(cudaMalloc(&d->mscales, sc.size()));
    CUDA_TRY(cudaMemcpy(d->mscales, sc.data(), sc.size(), cudaMemcpyHostToDevice));
    return 0;
}

/* Fill the mixed arenas from the host blocks (first use of mixed mode). */
static int pack_mixed(DevRep *d)
{
    if (d->arena32 != nullptr || d->arena32x2 != nullptr) return 0;
    std::vector<float> h32(std::max<size_t>(d->arena32_elems, 4), 0.f);
    std::vector<float2> h32x2(std::max<size_t>(d->arena32x2_elems, 2), make_float2(0.f, 0.f));
    for (const PackItem &it : d->mixed_items) {
        for (int r = 0; r < it.nrow; r++) {
            const double *src = it.src + (size_t)r * it.lds;
            for (int c = 0; c < it.ncol; c++) {
                /* position of source element (r, c) in the stored matrix */
                const size_t pos = it.off + (it.trans ? (size_t)c * it.ld + r : (size_t)r * it.ld + c);
                if (it.fmt == FMT_F32) {
                    h32[pos] = (float)src[c];
                } else {
                    /* float pairs: each 16-byte chunk (elements 2m, 2m+1 of a
                     * row) holds hi0, hi1, lo0, lo1, so the hi and lo parts of
                     * two neighbours are adjacent for packed arithmetic */
                    const float hi = (float)src[c];
                    float *f = reinterpret_cast<float *>(h32x2.data());
                    const size_t e = pos & ~size_t(1), k = pos & 1;
                    f[2 * e + k] = hi;
                    f[2 * e + 2 + k] = (float)(src[c] - (double)hi);
                }
            }
        }
    }
    CUDA_TRY(cudaMalloc(&d->arena32, h32.size() * sizeof(float)));
    CUDA_TRY(cudaMemcpy(d->arena32, h32.data(), h32.size() * sizeof(float), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMalloc(&d->arena32x2, h32x2.size() * sizeof(float2)));
    CUDA_TRY(cudaMemcpy(d->arena32x2, h32x2.data(), h32x2.size() * sizeof(float2), cudaMemcpyHostToDevice));
    int rc = mma_scales(d, h32, h32x2);
    if (rc) return rc;
    return build_tensor_maps(d);
}

int set_precision_mode(DevRep *d, H2ERI_p h, int mode)
{
    (void)h;
    if (mode == H2ERI_GPU_FP64 && d->arena == nullptr) {
        set_error("the FP64 copy of this structure was dropped (H2ERI_gpu_drop_fp64); release it "
                  "(H2ERI_gpu_release) and upload it again for the FP64 mode");
        return 3;
    }
    if (mode == H2ERI_GPU_MIXED) {
        int rc = pack_mixed(d);
        if (rc) return rc;
    }
    const bool changed = d->precision != mode;
    d->precision = mode;
    if (changed) {
        tune_apply_cached(d);   /* choices tuned earlier for this shape and precision */
        return apply_env_choices(d);
    }
    return 0;
}

/* ---- work list of the persistent kernel ---- */

static void px_free(DevRep *d)
{
    cudaFree(d->px.items);
    cudaFree(d->px.gneed);
    cudaFree(d->px.ctl);
    d->px = PxPlan();
}

/* Work list for nvec vectors: one item per (tile, vector), in the order a
 * list-scheduling simulation of the launch claims them. The simulation runs
 * `grid` workers, each streaming a tile at an equal share of the HBM rate
 * plus a fixed per-item cost; when a worker is free it takes the next tile
 * of the tree chain if that tile's preceding range is complete, else the
 * next ready near-field tile (the lane with more work left), else whichever
 * becomes ready first. Every queue is taken in its own order and a range's
 * items are only placed after all items of the range it depends on, so
 * the order is topological. */
static int build_px(DevRep *d, int nvec)
{
    if (d->px.items != nullptr && d->px.nvec == nvec) return 0;
    px_free(d);
    int occ = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_tile_px, kTileThreads, kPxSmem));
    if (occ < 1) {
        set_error("persistent tile kernel: no CTA fits on an SM");
        return 10;
    }
    /* ranges: the tree chain, then the near-field lanes */
    struct Grp { const Range *r; int dep; int queue; };
    std::vector<Grp> grp;
    int prev = -1;
    for (const std::vector<Range> *v : {&d->fwd, &d->mid, &d->bwd})
        for (const Range &r : *v) {
            if (r.count == 0) continue;
            grp.push_back({&r, prev, 0});
            prev = (int)grp.size() - 1;
        }
    int lane_prev[kNfLanes];
    for (int &x : lane_prev) x = -1;
    for (const Range &r : d->den) {
        if (r.count == 0) continue;
        const int ln = std::min(std::max(r.lane, 0), kNfLanes - 1);
        grp.push_back({&r, lane_prev[ln], 1 + ln});
        lane_prev[ln] = (int)grp.size() - 1;
    }
    const int ng = (int)grp.size();
    if (ng > 32000) { set_error("persistent tile kernel: too many ranges"); return 3; }
    const int nq = 1 + kNfLanes;
    std::vector<std::vector<PItem>> q(nq);
    std::vector<int> need(ng, 0);
    for (int g = 0; g < ng; g++) {
        const Range &r = *grp[g].r;
        for (int i = 0; i < r.count; i++)
            for (int v = 0; v < nvec; v++) {
                PItem it;
                it.tile = r.first + i;
                it.group = (int16_t)g;
                it.dep = (int16_t)grp[g].dep;
                it.v = (int16_t)v;
                it.fmt = (int16_t)(r.pair ? FMT_F32X2 : FMT_F32);
                it.pad_ = 0;
                q[grp[g].queue].push_back(it);
            }
        need[g] = r.count * nvec;
    }
    const int grid_max = occ * d->n_sm;
    /* simulation: seconds per byte of one worker, fixed cost per item */
    const double hbm = 6.0e12, per_item = 1.5e-6;
    const double spb = (double)grid_max / hbm;
    auto cost = [&](const PItem &it) {
        const Tile &t = d->tiles_host[it.tile];
        const double eb = it.fmt == FMT_F32 ? 4.0 : 8.0;
        return per_item + spb * (double)t.nr * (double)t.nc * eb;
    };
    const double INF = 1e300;
    std::vector<int> left(need);
    std::vector<double> fin(ng, 0.0);
    auto ready_at = [&](const PItem &it) { return it.dep < 0 ? 0.0 : (left[it.dep] ? INF : fin[it.dep]); };
    std::vector<size_t> head(nq, 0);
    std::vector<double> qleft(nq, 0.0);
    for (int k = 0; k < nq; k++)
        for (const PItem &it : q[k]) qleft[k] += cost(it);
    std::priority_queue<double, std::vector<double>, std::greater<double>> free_at;
    size_t total = 0;
    for (int k = 0; k < nq; k++) total += q[k].size();
    for (int w = 0; w < std::min<size_t>(grid_max, std::max<size_t>(total, 1)); w++) free_at.push(0.0);
    std::vector<PItem> order;
    order.reserve(total);
    double makespan = 0.0;
    while (order.size() < total) {
        const double T = free_at.top();
        free_at.pop();
        int pick = -1;
        if (head[0] < q[0].size() && ready_at(q[0][head[0]]) <= T) pick = 0;
        if (pick < 0)
            for (int j = 1; j < nq; j++)
                if (head[j] < q[j].size() && ready_at(q[j][head[j]]) <= T && (pick < 0 || qleft[j] > qleft[pick]))
                    pick = j;
        if (pick < 0) {
            double tb = INF;
            for (int k = 0; k < nq; k++)
                if (head[k] < q[k].size() && ready_at(q[k][head[k]]) < tb) { tb = ready_at(q[k][head[k]]); pick = k; }
        }
        if (pick < 0) { set_error("persistent tile kernel: schedule stalled"); return 3; }
        const PItem it = q[pick][head[pick]++];
        const double c = cost(it);
        const double t1 = std::max(T, ready_at(it)) + c;
        qleft[pick] -= c;
        fin[it.group] = std::max(fin[it.group], t1);
        left[it.group]--;
        makespan = std::max(makespan, t1);
        free_at.push(t1);
        order.push_back(it);
    }
    /* every item depends only on ranges whose items all come before it */
    {
        std::vector<int> seen(ng, 0);
        for (const PItem &it : order) {
            if (it.dep >= 0 && seen[it.dep] != need[it.dep]) {
                set_error("persistent tile kernel: work list is not in dependency order");
                return 3;
            }
            seen[it.group]++;
        }
    }
    PxPlan p;
    p.n_items = (int)order.size();
    p.n_groups = ng;
    p.ctl_ints = kPxDone + ng;
    p.nvec = nvec;
    p.grid = std::max(1, std::min(grid_max, p.n_items));
    p.sim_ms = makespan * 1e3;
    CUDA_TRY(cudaMalloc(&p.items, std::max<size_t>(order.size(), 1) * sizeof(PItem)));
    CUDA_TRY(cudaMalloc(&p.gneed, std::max(ng, 1) * sizeof(int)));
    CUDA_TRY(cudaMalloc(&p.ctl, p.ctl_ints * sizeof(int)));
    if (!order.empty())
        CUDA_TRY(cudaMemcpy(p.items, order.data(), order.size() * sizeof(PItem), cudaMemcpyHostToDevice));
    if (ng > 0) CUDA_TRY(cudaMemcpy(p.gneed, need.data(), ng * sizeof(int), cudaMemcpyHostToDevice));
    d->px = p;
    return 0;
}

/* The whole mixed single-density matvec as one persistent launch on s
 * (work and output already zeroed on s). A dependency wait gives up after
 * dep_limit cycles; 0 picks the default: about 1 s, or 20 times the
 * simulated duration of the launch if that is longer. */
static int launch_px(DevRep *d, const VecArgs &va, int nvec, cudaStream_t s, long long dep_limit = 0)
{
    int rc = build_px(d, nvec);
    if (rc) return rc;
    if (d->px.n_items == 0) return 0;
    if (dep_limit <= 0) dep_limit = std::max(2000000000LL, (long long)(d->px.sim_ms * 2.0e6 * 20.0));
    CUDA_TRY(cudaMemsetAsync(d->px.ctl, 0, d->px.ctl_ints * sizeof(int), s));
    k_tile_px<<<d->px.grid, kTileThreads, kPxSmem, s>>>(d->tiles, d->px.items, d->px.n_items, d->px.gneed,
                                                         d->px.ctl, va,
                                                         reinterpret_cast<const CUtensorMap *>(d->tmaps),
                                                         d->err_flag_dev, dep_limit);
    CUDA_TRY(cudaGetLastError());
    return 0;
}

/* The near field on its lanes: each lane (the float-pair blocks; groups of
 * single-float blocks) is an independent chain of three stages on its own
 * low-priority stream, so the few long CTAs at the end of one stage do not
 * leave the others waiting at a launch boundary. All lanes start after
 * ev_zero and are joined into s_aux, which records ev_join. */
static int launch_near_field(DevRep *d, const VecArgs &va, int nvec, bool timed = false, bool mma = false)
{
    for (int ln = 1; ln < kNfLanes; ln++) CUDA_TRY(cudaStreamWaitEvent(d->s_nf[ln], d->ev_zero, 0));
    CUDA_TRY(cudaStreamWaitEvent(d->s_aux, d->ev_zero, 0));
    for (size_t i = 0; i < d->den.size(); i++) {
        const Range &r = d->den[i];
        cudaStream_t ls = (r.lane == 0 || !d->cfg.nf_concurrent) ? d->s_aux : d->s_nf[r.lane];
        if (mma) launch_range_mma(d, d->mden[i], va, nvec, ls);
        else launch_range(d, r, va, nvec, ls);
    }
    for (int ln = 1; ln < kNfLanes; ln++) {
        CUDA_TRY(cudaEventRecord(d->ev_nf[ln], d->s_nf[ln]));
        CUDA_TRY(cudaStreamWaitEvent(d->s_aux, d->ev_nf[ln], 0));
    }
    if (timed) CUDA_TRY(cudaEventRecord(d->ev_t[7], d->s_aux));
    CUDA_TRY(cudaEventRecord(d->ev_join, d->s_aux));
    return 0;
}

/* Enqueue y = A x for nvec vectors (device pointers) on stream s. If timed,
 * per-phase events are recorded (fwd, mid, bwd on the main chain, dense on
 * the auxiliary stream). */
int enqueue_matvec(DevRep *d, int nvec, const double *x, double *y, cudaStream_t s, bool timed)
{
    /* an error an earlier runtime call left in this thread's error slot (and
     * handled where it happened) must not be reported as one of ours */
    (void)cudaGetLastError();
    int rc = ensure_work(d, nvec);
    if (rc) return rc;
    const size_t per_r = (size_t)d->rank_total * nvec, per_t = (size_t)d->lr_total * nvec;
    VecArgs va;
    std::memset(&va, 0, sizeof(va));
    va.base[VK_X] = const_cast<double *>(x);
    va.stride[VK_X] = d->krnl;
    va.base[VK_Y] = y;
    va.stride[VK_Y] = d->krnl;
    va.base[VK_Y0] = d->work;
    va.stride[VK_Y0] = d->rank_total;
    va.base[VK_Y1] = d->work + per_r;
    va.stride[VK_Y1] = d->rank_total;
    va.base[VK_T] = d->work + 2 * per_r;
    va.stride[VK_T] = d->lr_total;
    /* fork from the caller's stream onto the library's streams: the tree
     * chain on the high-priority stream, the near field on the other */
    cudaStream_t sm = d->s_main;
    CUDA_TRY(cudaEventRecord(d->ev_fork, s));
    CUDA_TRY(cudaStreamWaitEvent(sm, d->ev_fork, 0));
    CUDA_TRY(cudaMemsetAsync(d->work, 0, (2 * per_r + per_t) * sizeof(double), sm));
    CUDA_TRY(cudaMemsetAsync(y, 0, (size_t)d->krnl * nvec * sizeof(double), sm));
    CUDA_TRY(cudaEventRecord(d->ev_zero, sm));
    if (timed) CUDA_TRY(cudaEventRecord(d->ev_t[6], sm));
    /* several densities in the mixed mode: the tensor-core kernel, all
     * densities (up to 16 per pass) sharing each tile's slices */
    bool mma = d->precision == H2ERI_GPU_MIXED && nvec >= d->cfg.mma_min_vec;
    if (mma && d->mslices == nullptr) {
        rc = mma_make_slices(d);   /* first use of the tensor-core kernel */
        if (rc) return rc;
    }
    mma = mma && d->mslices != nullptr;
    if (d->precision == H2ERI_GPU_MIXED && !mma && d->cfg.persist) {
        /* one persistent launch: tree chain and near field from one work list */
        if (timed) for (int k : {0, 6}) CUDA_TRY(cudaEventRecord(d->ev_t[k], sm));
        rc = launch_px(d, va, nvec, sm);
        if (rc) return rc;
        if (timed) for (int k : {1, 2, 3, 7, 4}) CUDA_TRY(cudaEventRecord(d->ev_t[k], sm));
        CUDA_TRY(cudaEventRecord(d->ev_done, sm));
        CUDA_TRY(cudaStreamWaitEvent(s, d->ev_done, 0));
        CUDA_TRY(cudaGetLastError());
        return 0;
    }
    auto launch = [&](const Range &r) {
        if (mma) launch_range_mma(d, r, va, nvec, sm);
        else launch_range(d, r, va, nvec, sm);
    };
    rc = launch_near_field(d, va, nvec, timed, mma);
    if (rc) return rc;
    if (timed) CUDA_TRY(cudaEventRecord(d->ev_t[0], sm));
    for (const Range &r : (mma ? d->mfwd : d->fwd)) launch(r);
    if (timed) CUDA_TRY(cudaEventRecord(d->ev_t[1], sm));
    for (const Range &r : (mma ? d->mmid : d->mid)) launch(r);
    if (timed) CUDA_TRY(cudaEventRecord(d->ev_t[2], sm));
    for (const Range &r : (mma ? d->mbwd : d->bwd)) launch(r);
    if (timed) CUDA_TRY(cudaEventRecord(d->ev_t[3], sm));
    CUDA_TRY(cudaStreamWaitEvent(sm, d->ev_join, 0));
    if (timed) CUDA_TRY(cudaEventRecord(d->ev_t[4], sm));
    CUDA_TRY(cudaEventRecord(d->ev_done, sm));
    CUDA_TRY(cudaStreamWaitEvent(s, d->ev_done, 0));
    CUDA_TRY(cudaGetLastError());
    return 0;
}

/* After a synchronous call: a tile kernel that gave up a bounded wait for
 * a TMA load leaves a nonzero error word (mapped host memory). */
static int check_kernel_flag(DevRep *d)
{
    if (d->err_flag == nullptr || *d->err_flag == 0) return 0;
    const unsigned f = *d->err_flag;
    *d->err_flag = 0;
    if (f & 2u)
        set_error("a tile kernel found its shared memory off the 1024-byte alignment that swizzled TMA copies "
                  "need and did nothing; results are invalid");
    else if (f & 4u)
        set_error("the persistent tile kernel gave up waiting for a preceding range to complete (bounded wait "
                  "expired); results are invalid");
    else if (f & 8u)
        set_error("the exchange tensor-core kernel gave up waiting for its MMAs (bounded wait expired); results "
                  "are invalid");
    else
        set_error("a tile kernel gave up waiting for a TMA load (bounded wait expired); results are invalid");
    return 11;
}

/* After a timed enqueue has completed: fill the reference timers. */
static void collect_times(DevRep *d, H2ERI_p h)
{
    float f = 0, m = 0, b = 0, dn = 0, tot = 0;
    cudaEventElapsedTime(&f, d->ev_t[0], d->ev_t[1]);
    cudaEventElapsedTime(&m, d->ev_t[1], d->ev_t[2]);
    cudaEventElapsedTime(&b, d->ev_t[2], d->ev_t[3]);
    cudaEventElapsedTime(&dn, d->ev_t[6], d->ev_t[7]);
    cudaEventElapsedTime(&tot, d->ev_t[0], d->ev_t[4]);
    d->last_ms[0] = f; d->last_ms[1] = m; d->last_ms[2] = b; d->last_ms[3] = dn; d->last_ms[4] = tot;
    h->timers[MV_FWD_TIMER_IDX] += 1e-3 * f;
    h->timers[MV_MID_TIMER_IDX] += 1e-3 * m;
    h->timers[MV_BWD_TIMER_IDX] += 1e-3 * b;
    h->timers[MV_DEN_TIMER_IDX] += 1e-3 * dn;
    h->timers[MV_VOP_TIMER_IDX] += 1e-3 * std::max(0.0f, tot - (f + m + b));
}

static int ensure_den(DevRep *d, int n_den)
{
    if (n_den <= d->nden_cap) return 0;
    cudaFree(d->dbuf);
    cudaFree(d->jbuf);
    d->dbuf = d->jbuf = nullptr;
    size_t n2 = (size_t)d->num_bf * d->num_bf;
    CUDA_TRY(cudaMalloc(&d->dbuf, std::max<size_t>(n2 * n_den, 1) * sizeof(double)));
    CUDA_TRY(cudaMalloc(&d->jbuf, std::max<size_t>(n2 * n_den, 1) * sizeof(double)));
    d->nden_cap = n_den;
    return 0;
}

/* x = uncontracted densities (device arrays) into the structure's x buffer,
 * and J from its y buffer: the J-assembly launches of enqueue_coulomb, for
 * the merged batch path. */
int enqueue_uncontract(DevRep *d, int n_den, const double *den, cudaStream_t s)
{
    const long long n2 = (long long)d->num_bf * d->num_bf;
    dim3 g1((d->krnl + 255) / 256 < 4096 ? (d->krnl + 255) / 256 : 4096, n_den);
    k_uncontract<<<g1, 256, 0, s>>>(d->unc_map, d->krnl, den, n2, d->xbuf, d->krnl);
    CUDA_TRY(cudaGetLastError());
    return 0;
}
int enqueue_contract(DevRep *d, int n_den, double *J, cudaStream_t s)
{
    const long long n2 = (long long)d->num_bf * d->num_bf;
    long long nb = (n2 + 255) / 256;
    dim3 g2((unsigned)std::min<long long>(nb, 8192), n_den);
    k_contract<<<g2, 256, 0, s>>>(d->con_map, d->num_bf, d->ybuf, d->krnl, J, n2);
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int enqueue_coulomb(DevRep *d, int n_den, const double *den, double *J, cudaStream_t s, bool timed,
                    bool den_in_host)
{
    int rc = ensure_work(d, n_den);
    if (rc) return rc;
    const long long n2 = (long long)d->num_bf * d->num_bf;
    if (den_in_host) {
        dim3 g0((unsigned)std::min<long long>((n2 + 255) / 256, 8192), n_den);
        k_uncontract_scatter<<<g0, 256, 0, s>>>(d->con_map, n2, den, n2, d->xbuf, d->krnl);
    } else {
        dim3 g1((d->krnl + 255) / 256 < 4096 ? (d->krnl + 255) / 256 : 4096, n_den);
        k_uncontract<<<g1, 256, 0, s>>>(d->unc_map, d->krnl, den, n2, d->xbuf, d->krnl);
    }
    rc = enqueue_matvec(d, n_den, d->xbuf, d->ybuf, s, timed);
    if (rc) return rc;
    long long nb = (n2 + 255) / 256;
    dim3 g2((unsigned)std::min<long long>(nb, 8192), n_den);
    k_contract<<<g2, 256, 0, s>>>(d->con_map, d->num_bf, d->ybuf, d->krnl, J, n2);
    CUDA_TRY(cudaGetLastError());
    return 0;
}

}  // namespace h2g

using namespace h2g;

/* ======================================================================== */
/* C API                                                                     */
/* ======================================================================== */

[[noreturn]] static void fatal(const char *fn)
{
    std::fprintf(stderr, "[h2eri_gb300 FATAL] %s failed: %s\n", fn, t_last_error.c_str());
    std::fflush(stderr);
    std::abort();
}

extern "C" const char *H2ERI_gpu_last_error(void) { return t_last_error.c_str(); }

extern "C" int H2ERI_gpu_selftest_wait_timeout(long long cycles)
{
    if (cycles < 0) { set_error("cycles < 0"); return -1; }
    unsigned *flag = nullptr, *flag_dev = nullptr;
    if (cudaHostAlloc((void **)&flag, sizeof(unsigned), cudaHostAllocMapped) != cudaSuccess) {
        set_error(std::string("cudaHostAlloc: ") + cudaGetErrorString(cudaGetLastError()));
        return -1;
    }
    *flag = 0;
    int rc = -1;
    if (cudaHostGetDevicePointer((void **)&flag_dev, flag, 0) == cudaSuccess) {
        k_wait_probe<<<1, 32>>>(flag_dev, cycles);
        const cudaError_t e = cudaDeviceSynchronize();
        if (e == cudaSuccess) rc = *flag ? 1 : 0;
        else set_error(std::string("bounded-wait probe: ") + cudaGetErrorString(e));
    } else {
        set_error("cudaHostGetDevicePointer failed");
    }
    cudaFreeHost(flag);
    return rc;
}

/* The same bounded wait, enqueued on `stream` (NULL = the structure's own
 * stream) and reporting into the error word of a structure, the way the
 * mixed-mode tile kernels of the asynchronous entry points report: nothing is
 * checked here; H2ERI_gpu_check reports it afterwards. */
extern "C" int H2ERI_gpu_selftest_wait_timeout_async(H2ERI_p h2eri, long long cycles, void *stream)
{
    if (cycles < 0) { set_error("cycles < 0"); return 3; }
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : d->s_main;
    k_wait_probe<<<1, 32, 0, s>>>(d->err_flag_dev, cycles);
    CUDA_TRY(cudaGetLastError());
    return 0;
}

/* Failure-detection check of the persistent kernel's dependency waits: one
 * mixed single-density matvec of h2eri (zero input) with the item count of
 * its first range raised by one, so that the range after it waits for an
 * item that never completes. The wait gives up after `cycles`, the kernel
 * returns, and the expiry must be reported. The count is restored before
 * returning. Returns 1 when the expiry was reported, 0 when it was not, an
 * error code (> 1) otherwise. */
extern "C" int H2ERI_gpu_selftest_persist_timeout(H2ERI_p h2eri, long long cycles)
{
    if (cycles <= 0) { set_error("cycles must be > 0"); return 3; }
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return rc;
    if (d->precision != H2ERI_GPU_MIXED) { set_error("the persistent kernel runs in the mixed mode only"); return 3; }
    rc = ensure_work(d, 1);
    if (rc) return rc;
    rc = build_px(d, 1);
    if (rc) return rc;
    if (d->px.n_groups < 2) { set_error("the structure has a single range: nothing waits"); return 3; }
    CUDA_TRY(cudaDeviceSynchronize());
    (void)check_kernel_flag(d);   /* start from a clear record */
    int need0 = 0;
    CUDA_TRY(cudaMemcpy(&need0, d->px.gneed, sizeof(int), cudaMemcpyDeviceToHost));
    const int raised = need0 + 1;
    CUDA_TRY(cudaMemcpy(d->px.gneed, &raised, sizeof(int), cudaMemcpyHostToDevice));
    VecArgs va;
    std::memset(&va, 0, sizeof(va));
    const size_t per_r = (size_t)d->rank_total;
    va.base[VK_X] = d->xbuf; va.stride[VK_X] = d->krnl;
    va.base[VK_Y] = d->ybuf; va.stride[VK_Y] = d->krnl;
    va.base[VK_Y0] = d->work; va.stride[VK_Y0] = d->rank_total;
    va.base[VK_Y1] = d->work + per_r; va.stride[VK_Y1] = d->rank_total;
    va.base[VK_T] = d->work + 2 * per_r; va.stride[VK_T] = d->lr_total;
    cudaStream_t sm = d->s_main;
    int lrc = 0;
    if (cudaMemsetAsync(d->xbuf, 0, (size_t)d->krnl * sizeof(double), sm) != cudaSuccess ||
        cudaMemsetAsync(d->work, 0, (2 * per_r + d->lr_total) * sizeof(double), sm) != cudaSuccess ||
        cudaMemsetAsync(d->ybuf, 0, (size_t)d->krnl * sizeof(double), sm) != cudaSuccess)
        lrc = 10;
    if (lrc == 0) lrc = launch_px(d, va, 1, sm, cycles);
    const cudaError_t e = cudaStreamSynchronize(sm);
    CUDA_TRY(cudaMemcpy(d->px.gneed, &need0, sizeof(int), cudaMemcpyHostToDevice));
    if (lrc) return lrc;
    if (e != cudaSuccess) { set_error(std::string("persistent self-test: ") + cudaGetErrorString(e)); return 10; }
    const unsigned f = *d->err_flag;
    const int frc = check_kernel_flag(d);
    return (frc == 11 && (f & 4u)) ? 1 : 0;
}

/* Waits for the structure's own streams and reports what its kernels
 * recorded since the last check: an expired bounded wait (or a refused
 * shared-memory layout) in any kernel enqueued by the asynchronous entry
 * points (the _device variants, H2ERI_matvec_device_noalloc), which return
 * before their kernels run. Returns 0 when nothing was recorded, 11 (and
 * sets the message) otherwise; the record is cleared. The caller
 * synchronises its own stream first. */
extern "C" int H2ERI_gpu_check(H2ERI_p h2eri)
{
    if (h2eri == nullptr) { set_error("null H2ERI handle"); return 1; }
    DevRep *d = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_reps.find(h2eri);
        if (it == g_reps.end()) return 0;   /* nothing of it ever ran on the GPU */
        d = it->second;
    }
    CUDA_TRY(cudaStreamSynchronize(d->s_main));
    CUDA_TRY(cudaStreamSynchronize(d->s_aux));
    for (int i = 1; i < kNfLanes; i++) CUDA_TRY(cudaStreamSynchronize(d->s_nf[i]));
    return check_kernel_flag(d);
}

extern "C" int H2ERI_gpu_upload(H2ERI_p h2eri)
{
    DevRep *d;
    return get_rep(h2eri, &d);
}

/* Frees the FP64 copy of a structure that runs in the mixed mode (see the
 * header). Returns 0, 3 outside the mixed mode, or another error code. */
extern "C" int H2ERI_gpu_drop_fp64(H2ERI_p h2eri)
{
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return rc;
    if (d->precision != H2ERI_GPU_MIXED) {
        set_error("H2ERI_gpu_drop_fp64: the structure is not in the mixed mode");
        return 3;
    }
    if (d->arena == nullptr) return 0;
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(cudaFree(d->arena));
    d->arena = nullptr;
    return 0;
}

extern "C" void H2ERI_gpu_release(H2ERI_p h2eri)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_reps.find(h2eri);
    if (it == g_reps.end()) return;
    free_rep(it->second);
    g_reps.erase(it);
}

extern "C" int H2ERI_gpu_set_precision(H2ERI_p h2eri, int mode)
{
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return rc;
    if (mode != H2ERI_GPU_FP64 && mode != H2ERI_GPU_MIXED) {
        set_error("unknown precision mode");
        return 3;
    }
    return set_precision_mode(d, h2eri, mode);
}

extern "C" int H2ERI_matvec_device(H2ERI_p h2eri, int nvec, const double *d_x, double *d_y, void *stream)
{
    H2gRange nvtx_range("H2ERI_matvec_device");
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return rc;
    if (nvec < 1) { set_error("nvec < 1"); return 3; }
    cudaStream_t s = stream ? (cudaStream_t)stream : d->s_main;
    return enqueue_matvec(d, nvec, d_x, d_y, s, false);
}

extern "C" int H2ERI_matvec_multi(H2ERI_p h2eri, int nvec, const double *x, double *y)
{
    H2gRange nvtx_range("H2ERI_matvec_multi");
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return rc;
    if (nvec < 1) { set_error("nvec < 1"); return 3; }
    rc = ensure_work(d, nvec);
    if (rc) return rc;
    size_t bytes = (size_t)d->krnl * nvec * sizeof(double);
    CUDA_TRY(cudaMemcpyAsync(d->xbuf, x, bytes, cudaMemcpyHostToDevice, d->s_main));
    rc = enqueue_matvec(d, nvec, d->xbuf, d->ybuf, d->s_main, true);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(y, d->ybuf, bytes, cudaMemcpyDeviceToHost, d->s_main));
    CUDA_TRY(cudaStreamSynchronize(d->s_main));
    rc = check_kernel_flag(d);
    if (rc) return rc;
    collect_times(d, h2eri);
    h2eri->n_matvec += nvec;
    return 0;
}

extern "C" void H2ERI_matvec(H2ERI_p h2eri, const double *x, double *y)
{
    if (H2ERI_matvec_multi(h2eri, 1, x, y) != 0) fatal("H2ERI_matvec");
}

extern "C" int H2ERI_build_Coulomb_device(H2ERI_p h2eri, int n_den, const double *d_den, double *d_J, void *stream)
{
    H2gRange nvtx_range("H2ERI_build_Coulomb_device");
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return rc;
    if (n_den < 1) { set_error("n_den < 1"); return 3; }
    cudaStream_t s = stream ? (cudaStream_t)stream : d->s_main;
    return enqueue_coulomb(d, n_den, d_den, d_J, s, false);
}

/* J for several structures at once. In the mixed mode the H2 products of
 * all structures run in shared launches, one per phase, of the kernel their
 * launch choices name for their density count (h2g_batch.cu).
 * Otherwise every structure's build runs on its own pair of streams, forked
 * from `stream` and joined back to it, so the builds of small and large
 * molecules overlap on the GPU. All device buffers are set up before
 * anything is enqueued. */
extern "C" int H2ERI_build_Coulomb_batch(int n, H2ERI_p *h2eris, const int *n_den, const double *const *d_dens,
                                         double *const *d_Js, void *stream)
{
    H2gRange nvtx_range("H2ERI_build_Coulomb_batch");
    if (n < 0 || (n > 0 && (h2eris == nullptr || n_den == nullptr || d_dens == nullptr || d_Js == nullptr))) {
        set_error("H2ERI_build_Coulomb_batch: bad arguments");
        return 3;
    }
    std::vector<DevRep *> reps(n, nullptr);
    for (int i = 0; i < n; i++) {
        if (n_den[i] < 1) { set_error("H2ERI_build_Coulomb_batch: n_den < 1"); return 3; }
        for (int j = 0; j < i; j++)
            if (h2eris[j] == h2eris[i]) {
                set_error("H2ERI_build_Coulomb_batch: a structure appears twice (its builds share buffers)");
                return 3;
            }
        int rc = get_rep(h2eris[i], &reps[i]);
        if (rc) return rc;
        rc = ensure_work(reps[i], n_den[i]);
        if (rc) return rc;
    }
    cudaStream_t s = (cudaStream_t)stream;
    /* mixed mode with at most 16 densities per structure: every structure's
     * tiles in shared tensor-core launches, phase by phase */
    for (int i = 0; i < n; i++)   /* slices of the structures that will run the tensor-core kernel */
        if (reps[i]->precision == H2ERI_GPU_MIXED && n_den[i] >= reps[i]->cfg.mma_min_vec && n_den[i] <= 16) {
            const int rc = mma_make_slices(reps[i]);
            if (rc) return rc;
        }
    if (const int kind = batch_merged_kind(n, reps.data(), n_den))
        return batch_coulomb_merged(kind, n, reps.data(), n_den, d_dens, d_Js, s);
    for (int i = 0; i < n; i++) {
        DevRep *d = reps[i];
        CUDA_TRY(cudaEventRecord(d->ev_bfork, s));
        CUDA_TRY(cudaStreamWaitEvent(d->s_main, d->ev_bfork, 0));
        int rc = enqueue_coulomb(d, n_den[i], d_dens[i], d_Js[i], d->s_main, false);
        if (rc) return rc;
        CUDA_TRY(cudaEventRecord(d->ev_bjoin, d->s_main));
    }
    for (int i = 0; i < n; i++) CUDA_TRY(cudaStreamWaitEvent(s, reps[i]->ev_bjoin, 0));
    return 0;
}

/* Device address of a page-locked host buffer [p, p + bytes), or nullptr when
 * any part of it is pageable. Both ends must resolve to the same contiguous
 * device mapping, so kernels never reach host memory that is not mapped. */
static void *pinned_device_view(const void *p, size_t bytes)
{
    if (p == nullptr || bytes == 0) return nullptr;
    cudaPointerAttributes a0, a1;
    const char *last = static_cast<const char *>(p) + bytes - 1;
    if (cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || a0.devicePointer == nullptr ||
        a1.devicePointer == nullptr)
        return nullptr;
    if (static_cast<char *>(a1.devicePointer) - static_cast<char *>(a0.devicePointer) != (ptrdiff_t)(bytes - 1))
        return nullptr;
    return a0.devicePointer;
}

extern "C" int H2ERI_build_Coulomb_multi(H2ERI_p h2eri, int n_den, const double *den_mats, double *J_mats)
{
    H2gRange nvtx_range("H2ERI_build_Coulomb_multi");
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return rc;
    if (n_den < 1) { set_error("n_den < 1"); return 3; }
    size_t bytes = (size_t)d->num_bf * d->num_bf * n_den * sizeof(double);
    /* page-locked caller buffers are read and written in place over the
     * host link by the uncontract / contract kernels; pageable ones go
     * through device staging copies */
    const double *dsrc = static_cast<const double *>(pinned_device_view(den_mats, bytes));
    double *jdst = static_cast<double *>(pinned_device_view(J_mats, bytes));
    if (dsrc == nullptr || jdst == nullptr) {
        rc = ensure_den(d, n_den);
        if (rc) return rc;
    }
    if (dsrc == nullptr) {
        CUDA_TRY(cudaMemcpyAsync(d->dbuf, den_mats, bytes, cudaMemcpyHostToDevice, d->s_main));
        dsrc = d->dbuf;
    }
    rc = enqueue_coulomb(d, n_den, dsrc, jdst ? jdst : d->jbuf, d->s_main, true, dsrc != d->dbuf);
    if (rc) return rc;
    if (jdst == nullptr) CUDA_TRY(cudaMemcpyAsync(J_mats, d->jbuf, bytes, cudaMemcpyDeviceToHost, d->s_main));
    CUDA_TRY(cudaStreamSynchronize(d->s_main));
    rc = check_kernel_flag(d);
    if (rc) return rc;
    collect_times(d, h2eri);
    h2eri->n_matvec += n_den;
    return 0;
}

extern "C" void H2ERI_build_Coulomb(H2ERI_p h2eri, const double *den_mat, double *J_mat)
{
    if (H2ERI_build_Coulomb_multi(h2eri, 1, den_mat, J_mat) != 0) fatal("H2ERI_build_Coulomb");
}

extern "C" int H2ERI_gpu_report(H2ERI_p h2eri, double *out, int n)
{
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return -rc;
    int launches = 0;
    for (const Range &r : d->fwd) launches += r.count > 0;
    for (const Range &r : d->bwd) launches += r.count > 0;
    for (const Range &r : d->den) launches += r.count > 0;
    for (const Range &r : d->mid) launches += r.count > 0;
    /* the mixed single-density path with the persistent kernel: one launch */
    if (d->precision == H2ERI_GPU_MIXED && d->cfg.persist) launches = 1;
    double mbytes = d->precision == H2ERI_GPU_MIXED ? d->alg_bytes_matrix_mixed : d->alg_bytes_matrix;
    double vals[23] = {(double)launches, mbytes, d->alg_bytes_vec, d->alg_flops,
                       (double)d->bytes_U, (double)d->bytes_B, (double)d->bytes_D,
                       d->last_ms[0], d->last_ms[1], d->last_ms[2], d->last_ms[3], d->last_ms[4],
                       (double)d->precision, (double)(2.0 * d->rank_total + d->lr_total),
                       (double)d->cfg.chunk_rows, (double)d->cfg.tiles_per_cta, (double)d->cfg.nf_concurrent,
                       (double)d->cfg.mma_min_vec, (double)d->cfg.mma_grid_div, (double)d->cfg.persist,
                       (double)d->px.n_items, (double)d->px.grid, d->px.sim_ms};
    int m = std::min(n, 23);
    for (int i = 0; i < m; i++) out[i] = vals[i];
    return m;
}

extern "C" void h2g_gpu_print_statistic(H2ERI_p h2eri)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_reps.find(h2eri);
    if (it == g_reps.end()) return;
    DevRep *d = it->second;
    std::printf("==================== GPU (device %d) =======================\n", d->device);
    std::printf("  * Device arena U, B, D          : %.2lf, %.2lf, %.2lf (MB)\n", d->bytes_U / 1048576.0,
                d->bytes_B / 1048576.0, d->bytes_D / 1048576.0);
    std::printf("  * Tiles per matvec              : %d\n", d->n_tiles);
    if (d->last_ms[4] > 0)
        std::printf("  * Last matvec (ms) fwd/mid/bwd/dense/total : %.4f %.4f %.4f %.4f %.4f\n", d->last_ms[0],
                    d->last_ms[1], d->last_ms[2], d->last_ms[3], d->last_ms[4]);
}

/* ======================================================================== */
/* Matvec without allocation                                                 */
/* ======================================================================== */

namespace h2g {

/* Scratch of H2ERI_matvec_device_noalloc: the upward and downward
 * coefficients and the low-rank intermediates of one vector
 * (2 * rank_total + lr_total doubles; about 0.33 M for C30H62 at QR tol
 * 1e-8). 16 MiB, held by every GPU that loads this library until the process
 * exits. Every call uses the same array, and each call clears it before use,
 * so calls whose GPU work overlaps (different streams, or several structures
 * at once) race on it. */
constexpr size_t kNoAllocScratchDoubles = (size_t)1 << 21;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

static std::mutex g_noalloc_mu;
static std::unordered_map<int, double *> g_noalloc_addr;   /* device -> address of the array */

/* Device address of the scratch array on the current device. The host-side
 * name g_noalloc_scratch is only a stand-in and must never be passed to a
 * kernel; the address is looked up once per device, with that device
 * current, and cached. */
static int noalloc_scratch(int dev, double **out)
{
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    auto it = g_noalloc_addr.find(dev);
    if (it != g_noalloc_addr.end()) {
        *out = it->second;
        return 0;
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
        set_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        return 10;
    }
    g_noalloc_addr[dev] = static_cast<double *>(p);
    *out = static_cast<double *>(p);
    return 0;
}

}  // namespace h2g

/* Scratch limit of the allocation-free matvec: the array's size, or a lower
 * value from H2G_NOALLOC_LIMIT (doubles), which can only lower it. The lower
 * limit lets a caller (or a test) see the rejection of an oversized
 * representation without building one. */
static size_t noalloc_limit()
{
    size_t lim = kNoAllocScratchDoubles;
    if (const char *e = std::getenv("H2G_NOALLOC_LIMIT")) {
        char *end = nullptr;
        const unsigned long long v = std::strtoull(e, &end, 10);
        if (end != e && *end == '\0' && v < lim) lim = (size_t)v;
    }
    return lim;
}

/* y = A x for one vector on device arrays, without allocating device memory:
 * the representation must already be on the GPU (H2ERI_gpu_upload, or any
 * earlier hot-path call) and the intermediates use the library's fixed
 * scratch array. For callers that must not allocate after set-up: a host
 * application that hands the library a fixed device-memory budget, or one
 * whose memory pool is owned elsewhere, and latency-critical loops where
 * cudaMalloc/cudaFree would synchronise the device. The scratch array's
 * device address is looked up when the structure is uploaded, so this call
 * only reads it. A bounded-wait expiry inside the mixed-mode kernels is
 * reported by H2ERI_gpu_check after the stream has been synchronised. */
extern "C" int H2ERI_matvec_device_noalloc(H2ERI_p h2eri, const double *d_x, double *d_y, void *stream)
{
    H2gRange nvtx_range("H2ERI_matvec_device_noalloc");
    if (h2eri == nullptr) { set_error("null H2ERI handle"); return 1; }
    if (d_x == nullptr || d_y == nullptr) {
        set_error("H2ERI_matvec_device_noalloc: null input or output vector");
        return 3;
    }
    DevRep *d = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_reps.find(h2eri);
        if (it == g_reps.end()) {
            set_error("H2ERI_matvec_device_noalloc: no device copy of this structure; call H2ERI_gpu_upload first");
            return 2;
        }
        d = it->second;
        if (d->krnl != h2eri->krnl_mat_size || d->n_node != h2eri->n_node || d->fp_U != h2eri->U ||
            d->fp_B != h2eri->c_B_blks || d->fp_D != h2eri->c_D_blks) {
            set_error("H2ERI_matvec_device_noalloc: the structure changed since upload; call H2ERI_gpu_upload");
            return 2;
        }
    }
    const size_t need = (size_t)2 * d->rank_total + d->lr_total, limit = noalloc_limit();
    if (need > limit) {
        set_error("H2ERI_matvec_device_noalloc: needs " + std::to_string(need) + " doubles of scratch, limit " +
                  std::to_string(limit));
        return 4;
    }
    int dev = -1;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev != d->device) {
        set_error("H2ERI_matvec_device_noalloc: current device differs from the device holding the structure");
        return 5;
    }
    double *work = d->noalloc_work;
    if (work == nullptr) {
        set_error("H2ERI_matvec_device_noalloc: scratch address not resolved at upload");
        return 10;
    }

    const size_t per_r = (size_t)d->rank_total;
    VecArgs va;
    std::memset(&va, 0, sizeof(va));
    va.base[VK_X] = const_cast<double *>(d_x);
    va.stride[VK_X] = d->krnl;
    va.base[VK_Y] = d_y;
    va.stride[VK_Y] = d->krnl;
    va.base[VK_Y0] = work;
    va.stride[VK_Y0] = d->rank_total;
    va.base[VK_Y1] = work + per_r;
    va.stride[VK_Y1] = d->rank_total;
    va.base[VK_T] = work + 2 * per_r;
    va.stride[VK_T] = d->lr_total;
    cudaStream_t s = stream ? (cudaStream_t)stream : d->s_main;
    cudaStream_t sm = d->s_main;
    CUDA_TRY(cudaEventRecord(d->ev_fork, s));
    CUDA_TRY(cudaStreamWaitEvent(sm, d->ev_fork, 0));
    CUDA_TRY(cudaMemsetAsync(work, 0, need * sizeof(double), sm));      /* scratch keeps the last call's values */
    CUDA_TRY(cudaMemsetAsync(d_y, 0, (size_t)d->krnl * sizeof(double), sm));
    CUDA_TRY(cudaEventRecord(d->ev_zero, sm));
    const int rc = launch_near_field(d, va, 1);
    if (rc) return rc;
    for (const Range &r : d->fwd) launch_range(d, r, va, 1, sm);
    for (const Range &r : d->mid) launch_range(d, r, va, 1, sm);
    for (const Range &r : d->bwd) launch_range(d, r, va, 1, sm);
    CUDA_TRY(cudaStreamWaitEvent(sm, d->ev_join, 0));
    CUDA_TRY(cudaEventRecord(d->ev_done, sm));
    CUDA_TRY(cudaStreamWaitEvent(s, d->ev_done, 0));
    CUDA_TRY(cudaGetLastError());
    return 0;
}
