/*
 * GPU exchange (K) build, FP64.
 *
 * The reference (H2P-ERI src/H2ERI_build_exchange.c:1356-1450) forms K one
 * shell pair (N, Q) at a time: a partial H2 product with N_nbf * Q_nbf input
 * columns (q, n), input rows = the basis-function pairs (p, q) of the shell
 * pairs (P, Q) whose density block D[N, P] is significant (X[(p,q)][(q,n)] =
 * D[p][n]), output rows = the pairs (m, n) of the shell pairs (M, N), and
 * K[m][q] += sum_n Y[(m,n)][(q,n)]. Summed over all (N, Q) this is
 *
 *     K[m][q] = sum over stored rows r, columns c of A[r][c] * D'[p][n]
 *
 * where each stored basis-function pair (a in S1, b in S2) of a shell pair
 * (S1, S2) is read in both orientations (x, y) = (a, b) and (b, a) (one if
 * S1 == S2): (m, n) = (x, y) on the row side, (p, q) = (x, y) on the column
 * side, and D' is D with the insignificant (N, P) blocks zeroed (the
 * reference's dlist, :771-838).
 *
 * Here all (N, Q) are done at once, as batched dense products over the tree
 * (same blocks, same three coupling cases as the reference's partial
 * product, :1021-1353). Every node j carries the set S_j of basis functions
 * that occur in the pairs below it; for a range C of n:
 *   G_j[q][t][n] = sum_(p,q) below j  Ufull_j[(p,q)][t] D'[p][n]     q in S_j
 *   H_i[n][q][s] = sum_j B_ij G_j[q][.][n] + (from the parent)    n in S_i & C
 *   K[m][q]     += sum_(m,n) in leaf i  U_i[(m,n)] . H_i[n][q]
 * (G_j stored as [n][q][t] and H_i as [n][q][s]: the range index n outermost,
 * so a coupling product that reads G_j at the n of S_i reads whole contiguous
 * [q][t] slabs) which are the reference's forward transform (y0), coupling
 * (y1) and backward transform for all (N, Q) columns at once, restricted exactly as
 * the reference's row / column subtrees restrict them. The near-field blocks
 * are contracted directly. All contractions go through one gathered batched
 * FP64 GEMM kernel; K accumulates with FP64 atomics.
 */
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "h2eri_gb300.h"
#include "h2g_gpu_api.h"
#include "h2g_umma.cuh"

namespace h2g {

#define KCUDA_TRY(call)                                                                          \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                      \
            return 10;                                                                           \
        }                                                                                        \
    } while (0)

/* Significance threshold of a density block (src/H2ERI_build_exchange.c:784-806) */
constexpr double kDensityTol = 1e-10;

/* ======================================================================== */
/* Gathered batched GEMM                                                     */
/* ======================================================================== */

/* Operand element (r, c, z) = p[G(z) * sz + G(r) * sr + G(c) * sc], each G an
 * optional gather list (nullptr = identity). p points to doubles or floats
 * (the kernel's element type); c64 marks an FP64 output (K) of an FP32
 * product. */
struct Opnd {
    const void *p;
    const int *gr, *gc, *gz;
    long long sr, sc, sz;
};

/* C(i, (z, j)) += sum_k A(i, k) B(k, j, z), i < M, j < N, k < K, z < Z. The
 * batch index z is folded into the columns (column jz = z * N + j), so a tile
 * spans several batch entries when N is small; A does not depend on z. C is
 * updated with atomics (tasks of one launch may share outputs). */
struct GemmTask {
    Opnd a, b, c;
    int M, N, K, Z;
    int c64;
    int swap;   /* tensor-core kernel: tile rows are the product's columns (see k_gemm_tc) */
};

/* Tile shapes: FP64 64 x 64 (256 threads as 16 x 16, 4 x 4 per thread,
 * FP64-pipe bound), FP32 128 x 128 (512 threads as 16 x 32, 4 x 8 per
 * thread: twice the warps of an 8 x 8 layout, for more loads in flight).
 * k-steps of 16. */
template <typename T> struct GemmCfg;
template <> struct GemmCfg<double> { static constexpr int TM = 64, TN = 64, NT = 256; };
template <> struct GemmCfg<float> { static constexpr int TM = 128, TN = 128, NT = 512; };
constexpr int kGK = 16;
constexpr int kGThreads = 256;   /* threads of the FP64 variant */

template <typename T>
__host__ __device__ constexpr long long gemm_tiles(int M, int N, int Z)
{
    return (long long)((M + GemmCfg<T>::TM - 1) / GemmCfg<T>::TM) *
           (((long long)N * Z + GemmCfg<T>::TN - 1) / GemmCfg<T>::TN);
}

/* One CTA per TM x TN output tile; tile_start[t] is the first tile of task t
 * (prefix sums, tile_start[n_task] = total) and tile_task[tile] the task of a
 * tile. The operands are gathered
 * through index lists, so every k-step costs two dependent trips to L2
 * (index, then value): the indices are loaded two k-steps ahead and the
 * values one k-step ahead, both while the current step's FMAs run. */
template <typename T>
__global__ void __launch_bounds__(GemmCfg<T>::NT) k_gemm(const GemmTask *__restrict__ tasks,
                                                          const long long *__restrict__ tile_start, int n_task,
                                                          const int *__restrict__ tile_task)
{
    constexpr int TM = GemmCfg<T>::TM, TN = GemmCfg<T>::TN, NT = GemmCfg<T>::NT;
    constexpr int TY = NT / 16;                      /* thread rows */
    constexpr int RM = TM / TY, RN = TN / 16;
    constexpr int UA = TM * kGK / NT, UB = TN * kGK / NT;
    __shared__ T As[kGK][TM + 4];
    __shared__ T Bs[kGK][TN + 4];
    const long long tile = blockIdx.x;
    if (tile >= tile_start[n_task]) return;
    const int lo = tile_task[tile];
    const GemmTask &Tk = tasks[lo];
    const long long loc = tile - tile_start[lo];
    const long long NZ = (long long)Tk.N * Tk.Z;
    const long long tn_n = (NZ + TN - 1) / TN;
    const int m0 = (int)(loc / tn_n) * TM;
    const long long n0 = (loc % tn_n) * TN;
    const T *Ap = reinterpret_cast<const T *>(Tk.a.p);
    const T *Bp = reinterpret_cast<const T *>(Tk.b.p);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int K = Tk.K;

    /* operand offsets that stay fixed over k */
    const int ka = tid % kGK;                       /* k of this thread's A loads  */
    long long aro[UA];
#pragma unroll
    for (int u = 0; u < UA; u++) {
        int gi = m0 + (tid + u * NT) / kGK;
        aro[u] = gi < Tk.M ? (Tk.a.gr ? (long long)Tk.a.gr[gi] : (long long)gi) * Tk.a.sr : -1;
    }
    const int jb = tid % TN;                        /* column of this thread's B loads */
    long long bco;
    {
        long long jz = n0 + jb;
        if (jz < NZ) {
            int z = (int)(jz / Tk.N), c = (int)(jz % Tk.N);
            bco = (Tk.b.gz ? (long long)Tk.b.gz[z] : (long long)z) * Tk.b.sz +
                  (Tk.b.gc ? (long long)Tk.b.gc[c] : (long long)c) * Tk.b.sc;
        } else {
            bco = -1;
        }
    }
    /* gather offsets of one k-step: A column (one per thread), B rows */
    auto load_idx = [&](int k0, long long &ia, long long (&ib)[UB]) {
        const int gk = k0 + ka;
        ia = gk < K ? (Tk.a.gc ? (long long)Tk.a.gc[gk] : (long long)gk) * Tk.a.sc : -1;
#pragma unroll
        for (int u = 0; u < UB; u++) {
            const int gkb = k0 + (tid + u * NT) / TN;
            ib[u] = gkb < K ? (Tk.b.gr ? (long long)Tk.b.gr[gkb] : (long long)gkb) * Tk.b.sr : -1;
        }
    };
    auto load_val = [&](const long long ia, const long long (&ib)[UB], T (&ra)[UA], T (&rb)[UB]) {
#pragma unroll
        for (int u = 0; u < UA; u++) ra[u] = (aro[u] >= 0 && ia >= 0) ? Ap[aro[u] + ia] : T(0);
#pragma unroll
        for (int u = 0; u < UB; u++) rb[u] = (bco >= 0 && ib[u] >= 0) ? Bp[bco + ib[u]] : T(0);
    };

    T acc[RM][RN];
#pragma unroll
    for (int a = 0; a < RM; a++)
#pragma unroll
        for (int b = 0; b < RN; b++) acc[a][b] = T(0);

    long long ia0, ib0[UB], ia1, ib1[UB];
    T ra[UA], rb[UB];
    load_idx(0, ia0, ib0);
    load_idx(kGK, ia1, ib1);
    load_val(ia0, ib0, ra, rb);
    for (int k0 = 0; k0 < K; k0 += kGK) {
#pragma unroll
        for (int u = 0; u < UA; u++) As[ka][(tid + u * NT) / kGK] = ra[u];
#pragma unroll
        for (int u = 0; u < UB; u++) Bs[(tid + u * NT) / TN][jb] = rb[u];
        __syncthreads();
        /* next step's values (indices already here), the step after's indices */
        if (k0 + kGK < K) {
            load_val(ia1, ib1, ra, rb);
            ia0 = ia1;
#pragma unroll
            for (int u = 0; u < UB; u++) ib0[u] = ib1[u];
            load_idx(k0 + 2 * kGK, ia1, ib1);
        }
#pragma unroll
        for (int kk = 0; kk < kGK; kk++) {
            T av[RM], bv[RN];
#pragma unroll
            for (int a = 0; a < RM; a++) av[a] = As[kk][ty + TY * a];
#pragma unroll
            for (int b = 0; b < RN; b++) bv[b] = Bs[kk][tx + 16 * b];
#pragma unroll
            for (int a = 0; a < RM; a++)
#pragma unroll
                for (int b = 0; b < RN; b++) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
        }
        __syncthreads();
    }
    long long cco[RN];
#pragma unroll
    for (int b = 0; b < RN; b++) {
        long long jz = n0 + tx + 16 * b;
        if (jz < NZ) {
            int z = (int)(jz / Tk.N), c = (int)(jz % Tk.N);
            cco[b] = (Tk.c.gz ? (long long)Tk.c.gz[z] : (long long)z) * Tk.c.sz +
                     (Tk.c.gc ? (long long)Tk.c.gc[c] : (long long)c) * Tk.c.sc;
        } else {
            cco[b] = -1;
        }
    }
    /* output rows first (no index load waits behind the atomics) */
    long long cro[RM];
#pragma unroll
    for (int a = 0; a < RM; a++) {
        const int gi = m0 + ty + TY * a;
        cro[a] = gi < Tk.M ? (Tk.c.gr ? (long long)Tk.c.gr[gi] : (long long)gi) * Tk.c.sr : -1;
    }
    const bool c64 = Tk.c64 != 0;
    double *C64 = reinterpret_cast<double *>(const_cast<void *>(Tk.c.p));
    T *CT = reinterpret_cast<T *>(const_cast<void *>(Tk.c.p));
#pragma unroll
    for (int a = 0; a < RM; a++) {
        if (cro[a] < 0) continue;
#pragma unroll
        for (int b = 0; b < RN; b++) {
            if (cco[b] < 0) continue;
            if (c64) atomicAdd(C64 + cro[a] + cco[b], (double)acc[a][b]);
            else atomicAdd(CT + cro[a] + cco[b], acc[a][b]);
        }
    }
}

/* ======================================================================== */
/* The FP32 products on the tensor cores                                     */
/* ======================================================================== */

/* The mixed-mode products of k_gemm<float> as tcgen05 MMAs. Each FP32
 * operand element x is split exactly into three bf16 parts, x = h + m + l
 * (h, m, l: 8 + 8 + 8 significant bits, cut by truncation, see
 * tc_split2), and a tile accumulates the six products h h, and l h, m m, h l,
 * m h, h m in FP32 in tensor memory, h h in one accumulator and the five
 * smaller ones in a second (the tensor core's FP32 accumulation rounds
 * each MMA's sum, so h h gets the shortest chain; the two are added in
 * the epilogue); the three dropped products (m l, l m, l l) are below
 * 2^-24 |a b|, the rounding of FP32 accumulation (the bf16x3
 * scheme of G. Henry, P. T. P. Tang, A. Heinecke, "Leveraging the bfloat16
 * artificial intelligence datatype for higher-precision computations",
 * ARITH 2019).
 *
 * One CTA of 256 threads per 128 x 128 tile, two CTAs per SM. The tile's
 * rows are the TMEM lanes: the rows of C, or - for an output whose columns
 * are contiguous and rows are not (`swap`) - its columns, so that the
 * epilogue's atomics from consecutive lanes go to consecutive addresses.
 * Per 64-wide k step every thread gathers one row of each side (32 values
 * of each, through the task's index lists), splits them and stores the
 * slices into the 128-byte-swizzled K-major operand layout; one thread then
 * issues 4 x 6 MMAs of 128 x 128 x 16 and commits them to an mbarrier,
 * which the threads wait on (bounded, about a second) before they refill
 * the slices. After the last step the eight warps read the accumulator
 * (warp w: lanes 32 (w % 4) .., columns 64 (w / 4) ..) and add it to C with
 * FP32 or FP64 atomics. */
constexpr int kTcRows = 128;                          /* tile rows (TMEM lanes) = tile columns */
constexpr int kTcK = 64;                              /* k per step: one 128-byte row of bf16 */
constexpr int kTcThreads = 256;
constexpr uint32_t kTcSlice = kTcRows * kTcK * 2;     /* one bf16 slice of one side: 16 KB */
constexpr uint32_t kTcOffIdx = 6 * kTcSlice;          /* k offsets of both sides: 2 x 64 long long */
constexpr uint32_t kTcOffBar = kTcOffIdx + 2 * kTcK * 8;
constexpr uint32_t kTcSmem = kTcOffBar + 64;
constexpr uint32_t kTcSmemLaunch = kTcSmem + 1024;    /* + slack to align to 1024 bytes */
constexpr unsigned kTcErrBit = 8u;
constexpr uint32_t kTcTmemCols = 2 * kTcRows;         /* h h accumulator, then the corrections' */

__host__ __device__ constexpr long long tc_tiles(int M, int N, int Z)
{
    return (long long)((M + kTcRows - 1) / kTcRows) * (((long long)N * Z + kTcRows - 1) / kTcRows);
}

__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity)
{
    const long long t0 = clock64();
    uint32_t ok = 0;
    while (true) {
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok) return true;
        if (clock64() - t0 > 2000000000LL) return false;
    }
}

/* two FP32 values -> their h, m, l bf16 parts, packed low / high. The
 * parts are cut by truncation: h = the top 16 bits of x (sign, exponent, 7
 * fraction bits), m = the top 16 bits of x - h, l = x - h - m, which has at
 * most 8 significant bits left and so is a bf16 value too: x = h + m + l
 * exactly. */
__device__ __forceinline__ void tc_split2(float x0, float x1, uint32_t &h, uint32_t &m, uint32_t &l)
{
    const uint32_t b0 = __float_as_uint(x0), b1 = __float_as_uint(x1);
    h = __byte_perm(b0, b1, 0x7632);
    const float r0 = x0 - __uint_as_float(b0 & 0xFFFF0000u), r1 = x1 - __uint_as_float(b1 & 0xFFFF0000u);
    const uint32_t c0 = __float_as_uint(r0), c1 = __float_as_uint(r1);
    m = __byte_perm(c0, c1, 0x7632);
    const float t0 = r0 - __uint_as_float(c0 & 0xFFFF0000u), t1 = r1 - __uint_as_float(c1 & 0xFFFF0000u);
    l = __byte_perm(__float_as_uint(t0), __float_as_uint(t1), 0x7632);
}

/* Output of a tensor-core tile: the task's C operand held in registers. */
struct TcOut {
    void *p;
    const int *gr, *gc, *gz;
    long long sr, sc, sz, NZ;
    int M, N, c64, swap;
};

__device__ __forceinline__ TcOut tc_out(const GemmTask &Tk)
{
    TcOut o;
    o.p = const_cast<void *>(Tk.c.p);
    o.gr = Tk.c.gr; o.gc = Tk.c.gc; o.gz = Tk.c.gz;
    o.sr = Tk.c.sr; o.sc = Tk.c.sc; o.sz = Tk.c.sz;
    o.NZ = (long long)Tk.N * Tk.Z;
    o.M = Tk.M; o.N = Tk.N; o.c64 = Tk.c64; o.swap = Tk.swap;
    return o;
}

/* One warp's share of a tile epilogue: tile row mi (this lane) against the
 * 64 tile columns nj0 .. nj0 + 63 (those below Ne), accumulators at taddr
 * (h h) and taddr + 128 (corrections). The output offsets of the 64 columns
 * are formed first, two per lane, and handed around with shuffles, so that
 * no index load waits behind the atomics. With release != 0 the warp's
 * lane 0 arrives there once the accumulators are read. */
__device__ __forceinline__ void tc_epilogue(const TcOut &o, long long mi, long long nj0, long long Ne, uint32_t taddr,
                                            int lane, uint32_t release)
{
    auto col_off = [&](long long jz) -> long long {
        const int z = (int)jz / o.N, c = (int)jz - z * o.N;
        return (o.gz ? (long long)o.gz[z] : (long long)z) * o.sz + (o.gc ? (long long)o.gc[c] : (long long)c) * o.sc;
    };
    auto row_off = [&](long long i) -> long long { return (o.gr ? (long long)o.gr[i] : i) * o.sr; };
    const long long fc = o.swap ? (mi < o.NZ ? col_off(mi) : -1) : (mi < o.M ? row_off(mi) : -1);
    const long long j0a = nj0 + lane, j1a = nj0 + 32 + lane;
    const long long oc0 = j0a < Ne ? (o.swap ? row_off(j0a) : col_off(j0a)) : 0;
    const long long oc1 = j1a < Ne ? (o.swap ? row_off(j1a) : col_off(j1a)) : 0;
    const int nvalid = (int)max(0LL, min(64LL, Ne - nj0));
    double *C64 = reinterpret_cast<double *>(o.p);
    float *C32 = reinterpret_cast<float *>(o.p);
#pragma unroll 1
    for (int j0 = 0; j0 < 64; j0 += 16) {
        uint32_t rr[16], rc[16];
        umma::tmem_ld16(taddr + (uint32_t)j0, rr);
        umma::tmem_ld16(taddr + (uint32_t)(kTcRows + j0), rc);
        umma::tmem_wait_ld();
        if (release != 0 && j0 == 48) {
            umma::fence_before_sync();
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(release) : "memory");
        }
        if (j0 >= nvalid) continue;
        const long long ocs = j0 < 32 ? oc0 : oc1;
#pragma unroll
        for (int e = 0; e < 16; e++) {
            if (j0 + e >= nvalid) break;
            const long long o2 = __shfl_sync(0xffffffffu, ocs, (j0 + e) & 31);
            if (fc < 0) continue;
            const float v = __uint_as_float(rr[e]) + __uint_as_float(rc[e]);
            if (o.c64) atomicAdd(C64 + fc + o2, (double)v);
            else atomicAdd(C32 + fc + o2, v);
        }
    }
}

__global__ void __launch_bounds__(kTcThreads, 2) k_gemm_tc(const GemmTask *__restrict__ tasks,
                                                           const long long *__restrict__ tile_start, int n_task,
                                                           const int *__restrict__ tile_task, unsigned *err)
{
    extern __shared__ __align__(16) unsigned char tc_raw[];
    unsigned char *sm = tc_raw + ((1024u - (umma::smem_u32(tc_raw) & 1023u)) & 1023u);
    long long *kofs = reinterpret_cast<long long *>(sm + kTcOffIdx);   /* [side][k] */
    const uint32_t sbase = umma::smem_u32(sm), bar = sbase + kTcOffBar;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + kTcOffBar + 8);
    volatile int *dead = reinterpret_cast<volatile int *>(sm + kTcOffBar + 12);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    const long long tile = blockIdx.x;
    if (tile >= tile_start[n_task]) return;
    const int lo = tile_task[tile];
    const GemmTask &Tk = tasks[lo];
    const long long loc = tile - tile_start[lo];
    const bool swap = Tk.swap != 0;
    const long long NZ = (long long)Tk.N * Tk.Z;
    const long long Ne = swap ? (long long)Tk.M : NZ;
    const long long tn = (Ne + kTcRows - 1) / kTcRows;
    const long long m0 = (loc / tn) * kTcRows, n0 = (loc % tn) * kTcRows;
    const int K = Tk.K;

    /* offsets of a row of A, of a column of B and C (-1 past the extent) */
    auto a_row = [&](long long i) -> long long {
        return i < Tk.M ? (Tk.a.gr ? (long long)Tk.a.gr[i] : i) * Tk.a.sr : -1;
    };
    auto b_col = [&](long long jz) -> long long {
        if (jz >= NZ) return -1;
        const int z = (int)(jz / Tk.N), c = (int)(jz - (long long)z * Tk.N);
        return (Tk.b.gz ? (long long)Tk.b.gz[z] : (long long)z) * Tk.b.sz +
               (Tk.b.gc ? (long long)Tk.b.gc[c] : (long long)c) * Tk.b.sc;
    };
    /* side 0 fills the A operand of the MMA (tile rows), side 1 the B operand */
    const int r = tid & (kTcRows - 1), kh = tid >> 7;
    const float *Ap = reinterpret_cast<const float *>(Tk.a.p), *Bp = reinterpret_cast<const float *>(Tk.b.p);
    const float *sp[2] = {swap ? Bp : Ap, swap ? Ap : Bp};
    const long long sf[2] = {swap ? b_col(m0 + r) : a_row(m0 + r), swap ? a_row(n0 + r) : b_col(n0 + r)};

    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *dead = 0;
    }
    if (warp == 0) umma::tmem_alloc(tmem_slot, kTcTmemCols);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    const int nstep = (K + kTcK - 1) / kTcK;
    int issued = 0;
    for (int st = 0; st < nstep; st++) {
        const int k0 = st * kTcK;
        if (tid < 2 * kTcK) {
            /* A's k is its column (gc, sc), B's k is its row (gr, sr) */
            const int side = tid / kTcK, k = k0 + (tid % kTcK);
            const bool from_a = (side == 0) != swap;
            const int *kg = from_a ? Tk.a.gc : Tk.b.gr;
            const long long ks = from_a ? Tk.a.sc : Tk.b.sr;
            kofs[tid] = k < K ? (kg ? (long long)kg[k] : (long long)k) * ks : -1;
        }
        /* the slices of the previous step are free once its MMAs are done */
        if (issued > 0 && !tc_wait(bar, (uint32_t)((issued - 1) & 1))) {
            atomicOr(err, kTcErrBit);
            *dead = 1;
        }
        __syncthreads();
        if (*dead) break;
#pragma unroll
        for (int side = 0; side < 2; side++) {
            const float *p = side ? sp[1] : sp[0];
            const long long f = side ? sf[1] : sf[0];
            const long long *ko = kofs + side * kTcK + kh * 32;
            unsigned char *dst = sm + (uint32_t)side * 3u * kTcSlice;
            if (f < 0 || k0 + kh * 32 >= K) {
                /* a padding row, or k past the end: zero slices */
#pragma unroll
                for (int g = 0; g < 4; g++) {
                    const uint32_t off = umma::kmajor_off(r, kh * 32 + g * 8, 0);
                    const uint4 z = make_uint4(0, 0, 0, 0);
                    *reinterpret_cast<uint4 *>(dst + off) = z;
                    *reinterpret_cast<uint4 *>(dst + kTcSlice + off) = z;
                    *reinterpret_cast<uint4 *>(dst + 2 * kTcSlice + off) = z;
                }
                continue;
            }
            /* the 32 loads of this side first, then the splits */
            const float *pr = p + f;
            float v[32];
#pragma unroll
            for (int e = 0; e < 32; e++) {
                const long long o = ko[e];
                v[e] = o >= 0 ? pr[o] : 0.f;
            }
#pragma unroll
            for (int g = 0; g < 4; g++) {
                uint32_t hw[4], mw[4], lw[4];
#pragma unroll
                for (int e = 0; e < 4; e++) tc_split2(v[g * 8 + 2 * e], v[g * 8 + 2 * e + 1], hw[e], mw[e], lw[e]);
                const uint32_t off = umma::kmajor_off(r, kh * 32 + g * 8, 0);
                *reinterpret_cast<uint4 *>(dst + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(dst + kTcSlice + off) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
                *reinterpret_cast<uint4 *>(dst + 2 * kTcSlice + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
        }
        umma::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after_sync();
            const uint32_t idesc = umma::idesc_bf16(kTcRows, kTcRows, 0, 0);
            const uint32_t a0 = sbase, b0 = sbase + 3u * kTcSlice;
            const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
            const int nkk = min(kTcK / 16, (K - k0 + 15) / 16);   /* 16-wide k steps that hold data */
            for (int kk = 0; kk < nkk; kk++)
#pragma unroll
                for (int q = 0; q < 6; q++) {
                    const uint64_t ad = umma::sdesc(a0 + (uint32_t)pa[q] * kTcSlice + (uint32_t)kk * 32u, 16, 1024);
                    const uint64_t bd = umma::sdesc(b0 + (uint32_t)pb[q] * kTcSlice + (uint32_t)kk * 32u, 16, 1024);
                    /* q = 5 (h h) into columns [0, 128), the corrections into [128, 256) */
                    umma::mma_bf16(q == 5 ? tmem : tmem + kTcRows, ad, bd, idesc, st > 0 || kk > 0 || (q > 0 && q < 5));
                }
            umma::mma_commit(bar);
        }
        issued++;
    }
    if (issued > 0 && !*dead && !tc_wait(bar, (uint32_t)((issued - 1) & 1))) {
        atomicOr(err, kTcErrBit);
        *dead = 1;
    }
    __syncthreads();
    umma::fence_after_sync();
    if (issued > 0 && !*dead) {
        /* epilogue: lanes of the tile rows, 64 columns per warp */
        const int q = warp & 3, hcol = warp >> 2;
        const TcOut o = tc_out(Tk);
        tc_epilogue(o, m0 + 32 * q + lane, n0 + hcol * 64, Ne,
                    tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(hcol * 64), lane, 0u);
    } else if (issued > 0) {
        (void)tc_wait(bar, (uint32_t)((issued - 1) & 1));   /* MMAs still in flight: wait (bounded) before freeing */
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, kTcTmemCols);
}

/* Persistent, warp-specialised form of k_gemm_tc (the default): one CTA
 * per SM walks the launch's tiles (tile = blockIdx.x + i * gridDim.x), and
 * the three jobs of a tile run in different warps on different tiles at
 * once: two groups of four producer warps gather, split and store the
 * 64-wide k steps of alternate tiles into their own slot of slices (96 KB a
 * slot; two tiles' loads in flight), one thread issues its 24
 * MMAs into one of two accumulator buffers (256 TMEM columns each: h h,
 * then the corrections), and eight epilogue warps read the other buffer
 * and add it to C. Hand-overs go through mbarriers: full (producer warps
 * -> MMA), empty (MMA commit -> producers), acc_full (last commit of a tile
 * -> epilogue), acc_empty (epilogue warps -> MMA). Every wait is bounded
 * (about a second); on expiry the kernel sets the error bit, every role
 * stops at its next wait, the MMA thread waits (bounded) for its last
 * commit, and the tensor memory is freed. */
constexpr int kPpWarps = 8, kPeWarps = 8;
constexpr int kPThreads = 32 * (kPpWarps + 1 + kPeWarps);
constexpr uint32_t kPStage = 6 * kTcSlice;
constexpr uint32_t kPOffIdx = 2 * kPStage;                        /* k offsets: [stage][side][64] */
constexpr uint32_t kPOffBar = kPOffIdx + 2 * 2 * kTcK * 8;
constexpr uint32_t kPSmem = kPOffBar + 128;
constexpr uint32_t kPSmemLaunch = kPSmem + 1024;
constexpr uint32_t kPTmemCols = 512;                              /* two buffers of 256 */

/* the tile's task and corner; false past the launch's tiles */
struct TcTile {
    int task;
    bool swap;
    long long m0, n0, NZ, Ne;
};
__device__ __forceinline__ void tc_tile(long long tile, const GemmTask *__restrict__ tasks,
                                        const long long *__restrict__ tile_start, const int *__restrict__ tile_task,
                                        TcTile &t)
{
    t.task = tile_task[tile];
    const GemmTask &Tk = tasks[t.task];
    const long long loc = tile - tile_start[t.task];
    t.swap = Tk.swap != 0;
    t.NZ = (long long)Tk.N * Tk.Z;
    t.Ne = t.swap ? (long long)Tk.M : t.NZ;
    const long long tn = (t.Ne + kTcRows - 1) / kTcRows;
    t.m0 = (loc / tn) * kTcRows;
    t.n0 = (loc % tn) * kTcRows;
}

__global__ void __launch_bounds__(kPThreads, 1) k_gemm_tcp(const GemmTask *__restrict__ tasks,
                                                           const long long *__restrict__ tile_start, int n_task,
                                                           const int *__restrict__ tile_task, unsigned *err)
{
    extern __shared__ __align__(16) unsigned char tcp_raw[];
    unsigned char *sm = tcp_raw + ((1024u - (umma::smem_u32(tcp_raw) & 1023u)) & 1023u);
    long long *kofs = reinterpret_cast<long long *>(sm + kPOffIdx);   /* [stage][side][k] */
    const uint32_t sbase = umma::smem_u32(sm), bar0 = sbase + kPOffBar;
    auto full = [&](int st) { return bar0 + 8u * st; };
    auto empty = [&](int st) { return bar0 + 16u + 8u * st; };
    auto acc_full = [&](int b) { return bar0 + 32u + 8u * b; };
    auto acc_empty = [&](int b) { return bar0 + 48u + 8u * b; };
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + kPOffBar + 64);
    volatile int *dead = reinterpret_cast<volatile int *>(sm + kPOffBar + 68);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long ntiles = tile_start[n_task];

    if (tid == 0) {
        for (int i = 0; i < 2; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(full(i)), "r"(kPpWarps / 2) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(empty(i)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(acc_full(i)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(acc_empty(i)), "r"(kPeWarps) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *dead = 0;
    }
    if (warp == kPpWarps) umma::tmem_alloc(tmem_slot, kPTmemCols);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    auto wait = [&](uint32_t bar, uint32_t parity) -> bool {
        if (*dead) return false;
        if (tc_wait(bar, parity)) return true;
        atomicOr(err, kTcErrBit);
        *dead = 1;
        return false;
    };

    if (warp < kPpWarps) {
        /* ---- producers: two groups of four warps; group g fills slot g
         * with the k steps of the CTA's tiles of parity g, so that two
         * tiles' loads are in flight at once. Thread: row r of both sides. ---- */
        const int grp = warp >> 2, r = tid & (kTcRows - 1), s = grp;
        long long uses = 0;   /* fills of slot s so far */
        int j = 0;
        for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, j++) {
            if ((j & 1) != grp) continue;
            TcTile ti;
            tc_tile(tile, tasks, tile_start, tile_task, ti);
            const GemmTask &Tk = tasks[ti.task];
            const int K = Tk.K;
            const float *Ap = reinterpret_cast<const float *>(Tk.a.p), *Bp = reinterpret_cast<const float *>(Tk.b.p);
            auto a_row = [&](long long i) -> long long {
                return i < Tk.M ? (Tk.a.gr ? (long long)Tk.a.gr[i] : i) * Tk.a.sr : -1;
            };
            auto b_col = [&](long long jz) -> long long {
                if (jz >= ti.NZ) return -1;
                const int z = (int)jz / Tk.N, cc = (int)jz - z * Tk.N;
                return (Tk.b.gz ? (long long)Tk.b.gz[z] : (long long)z) * Tk.b.sz +
                       (Tk.b.gc ? (long long)Tk.b.gc[cc] : (long long)cc) * Tk.b.sc;
            };
            const float *sp0 = ti.swap ? Bp : Ap, *sp1 = ti.swap ? Ap : Bp;
            const long long sf0 = ti.swap ? b_col(ti.m0 + r) : a_row(ti.m0 + r);
            const long long sf1 = ti.swap ? a_row(ti.n0 + r) : b_col(ti.n0 + r);
            const int nstep = (K + kTcK - 1) / kTcK;
            bool stop = false;
            for (int st = 0; st < nstep; st++, uses++) {
                (void)wait(empty(s), (uint32_t)((uses & 1) ^ 1));
                const int k0 = st * kTcK;
                {
                    const int side = r >> 6, kk = r & (kTcK - 1), k = k0 + kk;
                    const bool from_a = (side == 0) != ti.swap;
                    const int *kg = from_a ? Tk.a.gc : Tk.b.gr;
                    const long long ks = from_a ? Tk.a.sc : Tk.b.sr;
                    kofs[(s * 2 + side) * kTcK + kk] = k < K ? (kg ? (long long)kg[k] : (long long)k) * ks : -1;
                }
                asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(32 * kPpWarps / 2) : "memory");
                if (*dead) { stop = true; break; }
                unsigned char *stage = sm + (uint32_t)s * kPStage;
#pragma unroll
                for (int part = 0; part < 4; part++) {
                    const int side = part >> 1, kh = part & 1;
                    const float *p = side ? sp1 : sp0;
                    const long long f = side ? sf1 : sf0;
                    const long long *ko = kofs + (s * 2 + side) * kTcK + kh * 32;
                    unsigned char *dst = stage + (uint32_t)side * 3u * kTcSlice;
                    if (f < 0 || k0 + kh * 32 >= K) {
#pragma unroll
                        for (int g = 0; g < 4; g++) {
                            const uint32_t off = umma::kmajor_off(r, kh * 32 + g * 8, 0);
                            const uint4 z = make_uint4(0, 0, 0, 0);
                            *reinterpret_cast<uint4 *>(dst + off) = z;
                            *reinterpret_cast<uint4 *>(dst + kTcSlice + off) = z;
                            *reinterpret_cast<uint4 *>(dst + 2 * kTcSlice + off) = z;
                        }
                        continue;
                    }
                    const float *pr = p + f;
                    float v[32];
#pragma unroll
                    for (int e = 0; e < 32; e++) {
                        const long long o = ko[e];
                        v[e] = o >= 0 ? pr[o] : 0.f;
                    }
#pragma unroll
                    for (int g = 0; g < 4; g++) {
                        uint32_t hw[4], mw[4], lw[4];
#pragma unroll
                        for (int e = 0; e < 4; e++)
                            tc_split2(v[g * 8 + 2 * e], v[g * 8 + 2 * e + 1], hw[e], mw[e], lw[e]);
                        const uint32_t off = umma::kmajor_off(r, kh * 32 + g * 8, 0);
                        *reinterpret_cast<uint4 *>(dst + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                        *reinterpret_cast<uint4 *>(dst + kTcSlice + off) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
                        *reinterpret_cast<uint4 *>(dst + 2 * kTcSlice + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
                    }
                }
                umma::fence_async_smem();
                __syncwarp();
                if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(full(s)) : "memory");
            }
            if (stop) break;
        }
    } else if (warp == kPpWarps) {
        /* ---- MMA issue: one thread ---- */
        long long used0 = 0, used1 = 0;   /* k steps consumed from each slot */
        int i = 0;
        uint32_t last_bar = 0, last_par = 0;
        bool any = false;
        const uint32_t idesc = umma::idesc_bf16(kTcRows, kTcRows, 0, 0);
        const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
        for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, i++) {
            TcTile ti;
            tc_tile(tile, tasks, tile_start, tile_task, ti);
            const int K = tasks[ti.task].K;
            const int b = i & 1;
            const uint32_t acc = tmem + (uint32_t)(b * 2 * kTcRows);
            bool ok = true;
            if (lane == 0) ok = wait(acc_empty(b), (uint32_t)(((i >> 1) & 1) ^ 1));
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            const int nstep = (K + kTcK - 1) / kTcK;
            const int s = i & 1;      /* the slot of the producer group of this tile's parity */
            const long long ub = s ? used1 : used0;
            if (s) used1 += nstep; else used0 += nstep;
            for (int st = 0; st < nstep; st++) {
                const uint32_t par = (uint32_t)((ub + st) & 1);
                if (lane == 0) ok = wait(full(s), par);
                ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
                if (!ok) break;
                if (lane == 0) {
                    umma::fence_after_sync();
                    const uint32_t a0 = sbase + (uint32_t)s * kPStage, b0 = a0 + 3u * kTcSlice;
                    const int nkk = min(kTcK / 16, (K - st * kTcK + 15) / 16);
                    for (int kk = 0; kk < nkk; kk++)
#pragma unroll
                        for (int q = 0; q < 6; q++) {
                            const uint64_t ad = umma::sdesc(a0 + (uint32_t)pa[q] * kTcSlice + (uint32_t)kk * 32u, 16, 1024);
                            const uint64_t bd = umma::sdesc(b0 + (uint32_t)pb[q] * kTcSlice + (uint32_t)kk * 32u, 16, 1024);
                            umma::mma_bf16(q == 5 ? acc : acc + kTcRows, ad, bd, idesc,
                                           st > 0 || kk > 0 || (q > 0 && q < 5));
                        }
                    umma::mma_commit(empty(s));
                    last_bar = empty(s);
                    last_par = par;
                    any = true;
                }
                __syncwarp();
            }
            if (!ok) break;
            if (lane == 0) {
                umma::mma_commit(acc_full(b));
                last_bar = acc_full(b);
                last_par = (uint32_t)((i >> 1) & 1);
            }
            __syncwarp();
        }
        /* after an expiry, MMAs may still be in flight: wait (bounded) for the last commit */
        if (lane == 0 && *dead && any) (void)tc_wait(last_bar, last_par);
    } else {
        /* ---- epilogue: 8 warps, lane quarter warp % 4, column half ---- */
        const int e = warp - kPpWarps - 1, q = warp & 3, hcol = e >> 2;
        int i = 0;
        for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, i++) {
            const int b = i & 1;
            bool ok = true;
            if (lane == 0) ok = wait(acc_full(b), (uint32_t)((i >> 1) & 1));
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            umma::fence_after_sync();
            TcTile ti;
            tc_tile(tile, tasks, tile_start, tile_task, ti);
            const TcOut o = tc_out(tasks[ti.task]);
            tc_epilogue(o, ti.m0 + 32 * q + lane, ti.n0 + hcol * 64, ti.Ne,
                        tmem + (uint32_t)(b * 2 * kTcRows) + ((uint32_t)(32 * q) << 16) + (uint32_t)(hcol * 64), lane,
                        acc_empty(b));
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == kPpWarps) umma::tmem_dealloc(tmem, kPTmemCols);
}

/* ======================================================================== */
/* Density screening and near field                                          */
/* ======================================================================== */

/* sig[N * nsh + P] = 1 if some |D[i][j]|, i in shell N, j in shell P, is above
 * the threshold (src/H2ERI_build_exchange.c:784-806). */
__global__ void k_density_sig(const double *__restrict__ den, int nbf, int nsh, const int *__restrict__ sb,
                              int *__restrict__ sig)
{
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)nsh * nsh) return;
    int N = (int)(t / nsh), P = (int)(t % nsh);
    int hit = 0;
    for (int i = sb[N]; i < sb[N + 1] && !hit; i++)
        for (int j = sb[P]; j < sb[P + 1]; j++)
            if (fabs(den[(long long)i * nbf + j]) > kDensityTol) { hit = 1; break; }
    sig[t] = hit;
}

/* D'[p][n] = D[p][n] if the block (shell(n), shell(p)) is significant, else 0:
 * the reference reads D[p][n] for P in dlist[N] only (:590-650). */
template <typename T>
__global__ void k_density_masked(const double *__restrict__ den, int nbf, int nsh, const int *__restrict__ bf_shell,
                                 const int *__restrict__ sig, T *__restrict__ dp)
{
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)nbf * nbf) return;
    int p = (int)(t / nbf), n = (int)(t % nbf);
    double v = sig[(long long)bf_shell[n] * nsh + bf_shell[p]] ? den[t] : 0.0;
    dp[t] = (T)v;
}

/* Near-field block use: rows = oriented pairs e of leaf i (local row, m, n),
 * columns = q-groups of leaf j (oriented pairs with the same q). Item (e, g):
 *   K[m_e][q_g] += sum_{f in g} Dblk(row_e, row_f) * D'[p_f][n_e]
 * with Dblk(r, c) = blk[r * ld + c], or blk[c * ld + r] when trans. */
struct NearTask {
    long long off;  /* element offset of the block in the arena */
    int ld, trans;
    int e0, ne;     /* oriented rows of leaf i: ext arrays [e0, e0 + ne) */
    int g0, ng;     /* q-groups of leaf j: group arrays [g0, g0 + ng)    */
};

struct ExtArrays {
    const int *row;   /* local row in the leaf                     */
    const int *x;     /* m on the row side, p on the column side    */
    const int *y;     /* n on the row side, q on the column side    */
    const int *gs;    /* group start (index into the ext arrays)    */
    const int *gc;    /* group count                                */
};

template <typename T>
__global__ void __launch_bounds__(256) k_near(const NearTask *__restrict__ tasks,
                                              const long long *__restrict__ item_start, int n_task, ExtArrays ex,
                                              const T *__restrict__ arena, const T *__restrict__ dp, int nbf,
                                              double *__restrict__ K)
{
    long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (it >= item_start[n_task]) return;
    int lo = 0, hi = n_task - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (item_start[mid] <= it) lo = mid; else hi = mid - 1;
    }
    const NearTask &Tk = tasks[lo];
    long long loc = it - item_start[lo];
    int e = Tk.e0 + (int)(loc / Tk.ng), g = Tk.g0 + (int)(loc % Tk.ng);
    const int re = ex.row[e], n = ex.y[e];
    const int f0 = ex.gs[g], nf = ex.gc[g];
    const T *blk = arena + Tk.off;
    const T *drow = dp + n;  /* D'[p][n] = drow[p * nbf] */
    T s = T(0);
    if (!Tk.trans) {
        const T *b = blk + (long long)re * Tk.ld;
        for (int f = f0; f < f0 + nf; f++) s = fma(b[ex.row[f]], drow[(long long)ex.x[f] * nbf], s);
    } else {
        for (int f = f0; f < f0 + nf; f++)
            s = fma(blk[(long long)ex.row[f] * Tk.ld + re], drow[(long long)ex.x[f] * nbf], s);
    }
    if (s != T(0)) atomicAdd(K + (long long)ex.x[e] * nbf + ex.y[f0], (double)s);
}

/* FP32 copies of the arena and of the masked density (mixed mode) */
__global__ void k_to_f32(const double *__restrict__ src, float *__restrict__ dst, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = __double2float_rn(src[i]);
}

/* ======================================================================== */
/* Plan                                                                      */
/* ======================================================================== */

/* Buffers a host-side operand refers to before device addresses exist. */
enum KBuf : int { KB_ARENA = 0, KB_GH = 1, KB_K = 2, KB_DP = 3, KB_FACT = 4 };

struct HOpnd {
    int buf = KB_ARENA;
    long long off = 0;
    long long gr = -1, gc = -1, gz = -1;   /* offsets into the int pool, -1 = identity */
    long long sr = 0, sc = 0, sz = 0;
};

struct HTask {
    HOpnd a, b, c;
    int M, N, K, Z;
};

struct KGroup {
    int t0 = 0, nt = 0;            /* task range */
    long long tiles = 0;
    const char *phase = "";
};

struct KChunk {
    int n0 = 0, nc = 0;
    size_t gh_elems = 0;
    std::vector<KGroup> groups;   /* launch order */
};

/* Launch data of one arithmetic precision (tile shapes differ). */
struct KVariant {
    GemmTask *tasks = nullptr;
    long long *tile_start = nullptr;   /* per group: nt + 1 prefix sums, concatenated */
    int *tile_task = nullptr;          /* per group: the task of each tile, concatenated */
    std::vector<long long> group_tile_off;
    std::vector<long long> group_pre;  /* offset of each group's prefix array, launch order */
    std::vector<long long> group_tiles;
};

struct KState {
    int nbf = 0, nsh = 0;
    double *arena = nullptr;      /* U (row-major, ld = rank), B and D dense (row-major, ld = ncol) */
    float *arena32 = nullptr;     /* FP32 copy (mixed mode, made on first use) */
    size_t arena_elems = 0;
    int *pool = nullptr;          /* every index list of the plan */
    std::vector<HTask> htasks;    /* host copy of the tasks (the FP32 variant is made from it) */
    KVariant v64, v32, vtc;        /* FP64, FP32 SIMT, FP32 on the tensor cores */
    int use_tc = 1;               /* mixed mode: 1 persistent tensor-core kernel, 2 one tile per CTA, 0 FP32 SIMT (H2G_K_TC) */
    int n_sm = 1;
    bool f32_ready = false;       /* FP32 arena, density buffer and the task list of use_tc uploaded */
    unsigned *err_dev = nullptr;  /* the structure's kernel error word (device address) */
    NearTask *near = nullptr;
    long long *near_start = nullptr;
    int n_near = 0;
    long long near_items = 0;
    ExtArrays ext{};
    int *sb = nullptr, *bf_shell = nullptr, *sig = nullptr;
    double *dp = nullptr, *gh = nullptr, *kbuf = nullptr;
    float *dp32 = nullptr;
    size_t gh_elems = 0;
    std::vector<KChunk> chunks;
    double flops = 0.0;           /* per K build */
    float last_ms = 0.f;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

void free_exchange_state(DevRep *d)
{
    KState *k = (KState *)d->kstate;
    if (k == nullptr) return;
    cudaFree(k->arena); cudaFree(k->arena32); cudaFree(k->pool); cudaFree(k->dp32);
    for (KVariant *v : {&k->v64, &k->v32, &k->vtc}) { cudaFree(v->tasks); cudaFree(v->tile_start); cudaFree(v->tile_task); }
    cudaFree(k->near); cudaFree(k->near_start);
    cudaFree(k->sb); cudaFree(k->bf_shell); cudaFree(k->sig);
    cudaFree(k->dp); cudaFree(k->gh); cudaFree(k->kbuf);
    if (k->ev0) cudaEventDestroy(k->ev0);
    if (k->ev1) cudaEventDestroy(k->ev1);
    delete k;
    d->kstate = nullptr;
}

namespace {

struct PlanBuilder {
    std::vector<int> pool;
    std::vector<HTask> tasks;

    long long put(const std::vector<int> &v)
    {
        long long o = (long long)pool.size();
        pool.insert(pool.end(), v.begin(), v.end());
        return o;
    }
    void add(const HTask &t)
    {
        if (t.M > 0 && t.N > 0 && t.K > 0 && t.Z > 0) tasks.push_back(t);
    }
};

int csr_find(const int *rowptr, const int *colidx, const int *val, int r, int c)
{
    for (int k = rowptr[r]; k < rowptr[r + 1]; k++)
        if (colidx[k] == c) return val[k];
    return 0;
}

}  // namespace

/* Host-side bounds check of one operand: every element the kernel can touch
 * for r < R, c < C, z < Z lies in [0, size), every gather index in the pool. */
static bool opnd_in_bounds(const HOpnd &o, int R, int C, int Z, size_t size, const std::vector<int> &pool)
{
    auto range = [&](long long g, int n, long long &lo, long long &hi) {
        if (g < 0) { lo = 0; hi = n - 1; return true; }
        if (g + n > (long long)pool.size()) return false;
        lo = hi = pool[g];
        for (int i = 1; i < n; i++) { lo = std::min<long long>(lo, pool[g + i]); hi = std::max<long long>(hi, pool[g + i]); }
        return true;
    };
    long long rl, rh, cl, ch, zl, zh;
    if (!range(o.gr, R, rl, rh) || !range(o.gc, C, cl, ch) || !range(o.gz, Z, zl, zh)) return false;
    if (rl < 0 || cl < 0 || zl < 0 || o.sr < 0 || o.sc < 0 || o.sz < 0 || o.off < 0) return false;
    long long hi = o.off + zh * o.sz + rh * o.sr + ch * o.sc;
    return hi < (long long)size;
}

/* Device task list and tile prefix sums of one precision: operands point
 * into the FP64 or the FP32 arena, density and work tensors; K stays FP64. */
template <typename T>
static int upload_variant(KState *ks, bool tc = false)
{
    KVariant &v = std::is_same<T, double>::value ? ks->v64 : (tc ? ks->vtc : ks->v32);
    auto base = [&](int buf) -> const void * {
        switch (buf) {
        case KB_ARENA: return std::is_same<T, double>::value ? (const void *)ks->arena : (const void *)ks->arena32;
        case KB_GH: return ks->gh;
        case KB_K: return ks->kbuf;
        default: return std::is_same<T, double>::value ? (const void *)ks->dp : (const void *)ks->dp32;
        }
    };
    auto conv = [&](const HOpnd &o) {
        Opnd r;
        const size_t es = o.buf == KB_K ? sizeof(double) : sizeof(T);
        r.p = (const char *)base(o.buf) + o.off * (long long)es;
        r.gr = o.gr >= 0 ? ks->pool + o.gr : nullptr;
        r.gc = o.gc >= 0 ? ks->pool + o.gc : nullptr;
        r.gz = o.gz >= 0 ? ks->pool + o.gz : nullptr;
        r.sr = o.sr; r.sc = o.sc; r.sz = o.sz;
        return r;
    };
    std::vector<GemmTask> dt(ks->htasks.size() + 1);
    for (size_t t = 0; t < ks->htasks.size(); t++) {
        const HTask &Tk = ks->htasks[t];
        dt[t].a = conv(Tk.a); dt[t].b = conv(Tk.b); dt[t].c = conv(Tk.c);
        dt[t].M = Tk.M; dt[t].N = Tk.N; dt[t].K = Tk.K; dt[t].Z = Tk.Z;
        dt[t].c64 = Tk.c.buf == KB_K;
        /* tensor-core tiles run along the output's contiguous dimension */
        const bool rows_contig = Tk.c.gr < 0 && Tk.c.sr == 1, cols_contig = Tk.c.gc < 0 && Tk.c.sc == 1;
        dt[t].swap = tc && !rows_contig && cols_contig;
    }
    std::vector<long long> pre;
    std::vector<int> ttask;
    v.group_pre.clear();
    v.group_tiles.clear();
    v.group_tile_off.clear();
    for (const KChunk &ch : ks->chunks)
        for (const KGroup &g : ch.groups) {
            v.group_pre.push_back((long long)pre.size());
            v.group_tile_off.push_back((long long)ttask.size());
            long long acc = 0;
            pre.push_back(0);
            for (int t = g.t0; t < g.t0 + g.nt; t++) {
                const HTask &Tk = ks->htasks[t];
                const long long nt = tc ? tc_tiles(Tk.M, Tk.N, Tk.Z) : gemm_tiles<T>(Tk.M, Tk.N, Tk.Z);
                acc += nt;
                pre.push_back(acc);
                if (acc <= 0x7fffffffLL) ttask.insert(ttask.end(), (size_t)nt, t - g.t0);
            }
            if (acc > 0x7fffffffLL) { set_error("exchange: launch too large"); return 4; }
            v.group_tiles.push_back(acc);
        }
    pre.push_back(0);
    ttask.push_back(0);
    KCUDA_TRY(cudaMalloc(&v.tile_task, ttask.size() * sizeof(int)));
    KCUDA_TRY(cudaMemcpy(v.tile_task, ttask.data(), ttask.size() * sizeof(int), cudaMemcpyHostToDevice));
    KCUDA_TRY(cudaMalloc(&v.tasks, dt.size() * sizeof(GemmTask)));
    KCUDA_TRY(cudaMemcpy(v.tasks, dt.data(), dt.size() * sizeof(GemmTask), cudaMemcpyHostToDevice));
    KCUDA_TRY(cudaMalloc(&v.tile_start, pre.size() * sizeof(long long)));
    KCUDA_TRY(cudaMemcpy(v.tile_start, pre.data(), pre.size() * sizeof(long long), cudaMemcpyHostToDevice));
    return 0;
}

/* FP32 arena, density and task list, made on the first mixed-mode K build. */
static int ensure_f32(KState *ks)
{
    if (ks->f32_ready) return 0;
    if (ks->arena32 == nullptr) {
        KCUDA_TRY(cudaMalloc(&ks->arena32, ks->arena_elems * sizeof(float)));
        k_to_f32<<<1216, 256>>>(ks->arena, ks->arena32, (long long)ks->arena_elems);
        KCUDA_TRY(cudaGetLastError());
    }
    if (ks->dp32 == nullptr) KCUDA_TRY(cudaMalloc(&ks->dp32, (size_t)ks->nbf * ks->nbf * sizeof(float)));
    KCUDA_TRY(cudaDeviceSynchronize());
    if (const char *e = std::getenv("H2G_K_TC")) ks->use_tc = std::min(2, std::max(0, std::atoi(e)));
    int dev = 0;
    KCUDA_TRY(cudaGetDevice(&dev));
    KCUDA_TRY(cudaDeviceGetAttribute(&ks->n_sm, cudaDevAttrMultiProcessorCount, dev));
    /* only the task list of the kernel in use (a large 3-D plan holds
     * millions of tasks) */
    KVariant &w = ks->use_tc ? ks->vtc : ks->v32;
    for (void *q : {(void *)w.tasks, (void *)w.tile_start, (void *)w.tile_task}) cudaFree(q);
    w.tasks = nullptr; w.tile_start = nullptr; w.tile_task = nullptr;
    if (ks->use_tc) {
        KCUDA_TRY(cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmemLaunch));
        KCUDA_TRY(cudaFuncSetAttribute(k_gemm_tcp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPSmemLaunch));
    }
    const int rc = upload_variant<float>(ks, ks->use_tc != 0);
    if (rc == 0) ks->f32_ready = true;
    return rc;
}

/* Default cap of the G / H work tensors (bytes, sized for FP64): with 40 %
 * of the free memory as the other bound. C30H62's mixed K build: 5 n ranges
 * under a 16 GB cap 238 ms, 3 ranges (25-32 GB) 227 ms, 2 ranges 228 ms, one
 * range (80 GB) 233 ms. */
constexpr double kWorkCap = 32e9;

/* free_bytes: device memory the G / H work tensors may be sized against;
 * upload = false builds and checks the plan on the host only. */
static int build_kplan(H2ERI_p h, KState *ks, size_t free_bytes, bool upload, double cap_bytes = kWorkCap)
{
    const auto tp0 = std::chrono::steady_clock::now();
    auto secs = [&]() { return std::chrono::duration<double>(std::chrono::steady_clock::now() - tp0).count(); };
    const bool verbose = [] { const char *v = std::getenv("H2G_KPLAN_VERBOSE"); return v && v[0] == '1'; }();
    const int nbf = h->num_bf, nsh = h->nshell, n_node = h->n_node, num_sp = h->num_sp;
    const int krnl = h->krnl_mat_size, nl = h->n_leaf_node, maxc = h->max_child;
    const int *sb = h->shell_bf_sidx;
    const int minl = h->min_adm_level, maxl = h->max_level;
    ks->nbf = nbf;
    ks->nsh = nsh;

    std::vector<int> rank(n_node), level(n_node), nch(n_node), coff(n_node, 0);
    for (int i = 0; i < n_node; i++) {
        rank[i] = h->U[i]->ncol;
        level[i] = h->node_level[i];
        nch[i] = h->n_child[i];
    }
    for (int p = 0; p < n_node; p++) {
        int off = 0;
        for (int k = 0; k < nch[p]; k++) {
            int c = h->children[p * maxc + k];
            coff[c] = off;
            off += rank[c];
        }
    }
    auto child = [&](int p, int k) { return h->children[p * maxc + k]; };
    auto has_far = [&](int j) { return level[j] >= minl && rank[j] > 0; };

    /* ---- arena: U compact row-major, B and D dense; low-rank blocks are
     * expanded on the device (one GEMM task each, factors in a temporary
     * buffer), because the density coupling of K does not factor ---- */
    std::vector<size_t> uoff(n_node), boff(std::max(h->n_B, 1)), doff(std::max(h->n_D, 1));
    size_t tot = 0;
    for (int i = 0; i < n_node; i++) { uoff[i] = tot; tot += (size_t)h->U[i]->nrow * rank[i]; }
    for (int b = 0; b < h->n_B; b++) { boff[b] = tot; tot += (size_t)h->c_B_blks[b]->nrow * h->c_B_blks[b]->ncol; }
    for (int b = 0; b < h->n_D; b++) { doff[b] = tot; tot += (size_t)h->c_D_blks[b]->nrow * h->c_D_blks[b]->ncol; }
    const size_t arena_elems = tot + 1;
    std::vector<HTask> expand;
    std::vector<size_t> fact_off;
    size_t fact_elems = 0;
    auto plan_expand = [&](H2E_dense_mat_p m, size_t dst) {
        if (m->ld >= 0 || m->nrow == 0 || m->ncol == 0) return;
        const int r = -m->ld;
        HTask t{};
        t.M = m->nrow; t.N = m->ncol; t.K = r; t.Z = 1;
        t.a.buf = KB_FACT; t.a.off = (long long)fact_elems; t.a.sr = r; t.a.sc = 1;
        t.b.buf = KB_FACT; t.b.off = (long long)(fact_elems + (size_t)m->nrow * r); t.b.sr = 1; t.b.sc = r;
        t.c.buf = KB_ARENA; t.c.off = (long long)dst; t.c.sr = m->ncol; t.c.sc = 1;
        if (r > 0) expand.push_back(t);
        fact_off.push_back(fact_elems);
        fact_elems += (size_t)(m->nrow + m->ncol) * r;
    };
    for (int b = 0; b < h->n_B; b++) plan_expand(h->c_B_blks[b], boff[b]);
    for (int b = 0; b < h->n_D; b++) plan_expand(h->c_D_blks[b], doff[b]);

    /* ---- oriented rows of every leaf, grouped by their second index ---- */
    std::vector<int> row_sp(krnl + 1, 0);
    for (int sp = 0; sp < num_sp; sp++)
        for (int r = h->sp_bfp_sidx[sp]; r < h->sp_bfp_sidx[sp + 1]; r++) row_sp[r] = sp;
    std::vector<int> ext_off(n_node, 0), ext_cnt(n_node, 0), grp_off(n_node, 0), grp_cnt(n_node, 0);
    std::vector<int> e_row, e_x, e_y, g_start, g_cnt, g_y;
    std::vector<std::vector<int>> S(n_node);
    struct Ext { int y, x, row; };
    for (int li = 0; li < nl; li++) {
        const int L = h->height_nodes[li];
        const int r0 = h->mat_cluster[2 * L], r1 = h->mat_cluster[2 * L + 1];
        std::vector<Ext> v;
        v.reserve((size_t)2 * (r1 - r0 + 1));
        for (int r = r0; r <= r1; r++) {
            int sp = row_sp[r], idx = r - h->sp_bfp_sidx[sp];
            int S1 = h->sp_shell_idx[sp], S2 = h->sp_shell_idx[sp + num_sp];
            int n1 = sb[S1 + 1] - sb[S1];
            int a = sb[S1] + idx % n1, b = sb[S2] + idx / n1;
            v.push_back({b, a, r - r0});
            if (S1 != S2) v.push_back({a, b, r - r0});
        }
        std::sort(v.begin(), v.end(), [](const Ext &p, const Ext &q) {
            return p.y != q.y ? p.y < q.y : (p.x != q.x ? p.x < q.x : p.row < q.row);
        });
        ext_off[L] = (int)e_row.size();
        ext_cnt[L] = (int)v.size();
        grp_off[L] = (int)g_start.size();
        for (size_t k = 0; k < v.size();) {
            size_t k1 = k;
            while (k1 < v.size() && v[k1].y == v[k].y) k1++;
            g_start.push_back(ext_off[L] + (int)k);
            g_cnt.push_back((int)(k1 - k));
            g_y.push_back(v[k].y);
            S[L].push_back(v[k].y);
            k = k1;
        }
        grp_cnt[L] = (int)g_start.size() - grp_off[L];
        for (const Ext &e : v) { e_row.push_back(e.row); e_x.push_back(e.x); e_y.push_back(e.y); }
    }
    /* S of inner nodes: union of the children's, deepest level first */
    for (int lv = maxl; lv >= 0; lv--)
        for (int k = 0; k < h->level_n_node[lv]; k++) {
            int p = h->level_nodes[lv * nl + k];
            if (nch[p] == 0) continue;
            std::vector<int> u;
            for (int c = 0; c < nch[p]; c++) u.insert(u.end(), S[child(p, c)].begin(), S[child(p, c)].end());
            std::sort(u.begin(), u.end());
            u.erase(std::unique(u.begin(), u.end()), u.end());
            S[p].swap(u);
        }
    auto pos_in = [](const std::vector<int> &v, int x) {
        return (int)(std::lower_bound(v.begin(), v.end(), x) - v.begin());
    };

    const double t_sets = secs();
    PlanBuilder pb;
    const long long P_row = pb.put(e_row), P_x = pb.put(e_x);
    (void)pb.put(e_y);
    const long long P_gs = pb.put(g_start), P_gc = pb.put(g_cnt);
    const long long P_ey = P_x + (long long)e_x.size();
    std::vector<long long> P_S(n_node, -1), P_qmap(n_node, -1);
    for (int j = 0; j < n_node; j++) P_S[j] = pb.put(S[j]);
    for (int p = 0; p < n_node; p++)
        for (int k = 0; k < nch[p]; k++) {
            int c = child(p, k);
            std::vector<int> m(S[c].size());
            for (size_t t = 0; t < S[c].size(); t++) m[t] = pos_in(S[p], S[c][t]);
            P_qmap[c] = pb.put(m);
        }

    /* ---- near field: every (leaf, inadmissible partner) of the reference's lists (:1307-1350) ---- */
    std::vector<NearTask> hnear;
    std::vector<long long> near_pre(1, 0);
    double flops = 0.0;
    for (int li = 0; li < nl; li++) {
        const int i = h->height_nodes[li];
        for (int k = h->node_inadm_pairs_sidx[i]; k < h->node_inadm_pairs_sidx[i + 1]; k++) {
            int j = h->node_inadm_pairs[k];
            int pi = csr_find(h->D_p2i_rowptr, h->D_p2i_colidx, h->D_p2i_val, i, j);
            if (pi == 0) { set_error("exchange plan: missing near-field block"); return 2; }
            int di = (pi > 0 ? pi : -pi) - 1;
            if (ext_cnt[i] == 0 || grp_cnt[j] == 0) continue;
            NearTask t;
            t.off = (long long)doff[di];
            t.ld = h->c_D_blks[di]->ncol;
            t.trans = pi < 0;
            t.e0 = ext_off[i]; t.ne = ext_cnt[i];
            t.g0 = grp_off[j]; t.ng = grp_cnt[j];
            hnear.push_back(t);
            near_pre.push_back(near_pre.back() + (long long)t.ne * t.ng);
            flops += 2.0 * t.ne * (double)ext_cnt[j];
        }
    }

    /* ---- n ranges: keep G + H under a fixed share of the free device memory ---- */
    double full = 0.0;
    for (int j = 0; j < n_node; j++)
        if (has_far(j)) full += 2.0 * (double)S[j].size() * rank[j] * nbf;
    const double budget = std::max(1e6, std::min(cap_bytes, 0.4 * (double)free_bytes) / sizeof(double));
    int nchunk = (int)std::ceil(full / budget);
    nchunk = std::max(1, std::min(nchunk, nbf));

    std::vector<int> lvl_nodes_flat;
    auto level_list = [&](int lv) {
        std::vector<int> v;
        for (int k = 0; k < h->level_n_node[lv]; k++) v.push_back(h->level_nodes[lv * nl + k]);
        return v;
    };
    auto beff = [&](int b, bool trans, HOpnd &o) {   /* Beff(i, k): i on the row node's side */
        o.buf = KB_ARENA;
        o.off = (long long)boff[b];
        long long ncb = h->c_B_blks[b]->ncol;
        if (!trans) { o.sr = ncb; o.sc = 1; } else { o.sr = 1; o.sc = ncb; }
    };

    for (int c = 0; c < nchunk; c++) {
        KChunk ch;
        ch.n0 = (int)((long long)c * nbf / nchunk);
        int n1 = (int)((long long)(c + 1) * nbf / nchunk);
        ch.nc = n1 - ch.n0;
        const int n0 = ch.n0, nc = ch.nc;
        std::vector<long long> goff(n_node, -1), hoff(n_node, -1), P_sic(n_node, -1), P_sicl(n_node, -1);
        std::vector<std::vector<int>> sic(n_node);
        size_t e = 0;
        for (int j = 0; j < n_node; j++)
            if (has_far(j)) { goff[j] = (long long)e; e += S[j].size() * (size_t)rank[j] * nc; }
        for (int i = 0; i < n_node; i++) {
            if (!has_far(i)) continue;
            for (int x : S[i]) if (x >= n0 && x < n1) sic[i].push_back(x);
            std::vector<int> loc(sic[i]);
            for (int &x : loc) x -= n0;
            P_sic[i] = pb.put(sic[i]);
            P_sicl[i] = pb.put(loc);
            hoff[i] = (long long)e;
            e += sic[i].size() * (size_t)nbf * rank[i];
        }
        ch.gh_elems = e;
        auto open_group = [&](const char *ph) {
            KGroup g;
            g.t0 = (int)pb.tasks.size();
            g.phase = ph;
            ch.groups.push_back(g);
        };
        auto close_group = [&]() {
            KGroup &g = ch.groups.back();
            g.nt = (int)pb.tasks.size() - g.t0;
            if (g.nt == 0) ch.groups.pop_back();
        };

        /* forward, leaves: G_j[q] = U_j[rows with q]^T D'[p of those rows][C] (:1101-1155) */
        open_group("fwd-leaf");
        for (int li = 0; li < nl; li++) {
            const int j = h->height_nodes[li];
            if (!has_far(j)) continue;
            for (int g = grp_off[j]; g < grp_off[j] + grp_cnt[j]; g++) {
                HTask t{};
                t.M = rank[j]; t.N = nc; t.K = g_cnt[g]; t.Z = 1;
                t.a.buf = KB_ARENA; t.a.off = (long long)uoff[j]; t.a.sr = 1;
                t.a.gc = P_row + g_start[g]; t.a.sc = rank[j];
                t.b.buf = KB_DP; t.b.off = n0; t.b.gr = P_x + g_start[g]; t.b.sr = nbf; t.b.sc = 1;
                t.c.buf = KB_GH; t.c.off = goff[j] + (long long)pos_in(S[j], g_y[g]) * rank[j];
                t.c.sr = 1; t.c.sc = (long long)S[j].size() * rank[j];
                pb.add(t);
            }
        }
        close_group();
        /* forward, inner nodes: G_p[q] += E_c^T G_c[q], level by level */
        for (int lv = maxl - 1; lv >= minl; lv--) {
            open_group("fwd-inner");
            for (int p : level_list(lv)) {
                if (nch[p] == 0 || !has_far(p)) continue;
                for (int k = 0; k < nch[p]; k++) {
                    int cc = child(p, k);
                    if (!has_far(cc)) continue;
                    HTask t{};
                    t.M = rank[p]; t.N = nc; t.K = rank[cc]; t.Z = (int)S[cc].size();
                    t.a.buf = KB_ARENA; t.a.off = (long long)uoff[p] + (long long)coff[cc] * rank[p];
                    t.a.sr = 1; t.a.sc = rank[p];
                    t.b.buf = KB_GH; t.b.off = goff[cc]; t.b.sr = 1; t.b.sc = (long long)S[cc].size() * rank[cc];
                    t.b.sz = rank[cc];
                    t.c.buf = KB_GH; t.c.off = goff[p]; t.c.sr = 1; t.c.sc = (long long)S[p].size() * rank[p];
                    t.c.gz = P_qmap[cc]; t.c.sz = rank[p];
                    pb.add(t);
                }
            }
            close_group();
        }

        /* coupling blocks, the three level cases of the partial product (:1160-1250) */
        open_group("coupling");
        for (int i = 0; i < n_node; i++) {
            for (int k = h->node_adm_pairs_sidx[i]; k < h->node_adm_pairs_sidx[i + 1]; k++) {
                const int j = h->node_adm_pairs[k];
                int pi = csr_find(h->B_p2i_rowptr, h->B_p2i_colidx, h->B_p2i_val, i, j);
                if (pi == 0) { set_error("exchange plan: missing coupling block"); return 2; }
                const bool tr = pi < 0;
                const int b = (tr ? -pi : pi) - 1;
                if (level[i] == level[j]) {
                    /* H_i[n][q] += Beff G_j[q][.][n]   (n in S_i & C, q in S_j) */
                    if (rank[i] == 0 || rank[j] == 0 || sic[i].empty() || !has_far(i) || !has_far(j)) continue;
                    HTask t{};
                    t.M = rank[i]; t.N = (int)sic[i].size(); t.K = rank[j]; t.Z = (int)S[j].size();
                    beff(b, tr, t.a);
                    t.b.buf = KB_GH; t.b.off = goff[j]; t.b.sr = 1; t.b.gc = P_sicl[i];
                    t.b.sc = (long long)S[j].size() * rank[j]; t.b.sz = rank[j];
                    t.c.buf = KB_GH; t.c.off = hoff[i]; t.c.sr = 1; t.c.sc = (long long)nbf * rank[i];
                    t.c.gz = P_S[j]; t.c.sz = rank[i];
                    pb.add(t);
                } else if (level[i] > level[j]) {
                    /* j is a leaf above i: H_i[n][q] += Beff[., rows of q] D'[p][n] */
                    if (!has_far(i) || sic[i].empty()) continue;
                    for (int g = grp_off[j]; g < grp_off[j] + grp_cnt[j]; g++) {
                        HTask t{};
                        t.M = rank[i]; t.N = (int)sic[i].size(); t.K = g_cnt[g]; t.Z = 1;
                        beff(b, tr, t.a);
                        t.a.gc = P_row + g_start[g];
                        t.b.buf = KB_DP; t.b.off = 0; t.b.gr = P_x + g_start[g]; t.b.sr = nbf;
                        t.b.gc = P_sic[i]; t.b.sc = 1;
                        t.c.buf = KB_GH; t.c.off = hoff[i] + (long long)g_y[g] * rank[i];
                        t.c.sr = 1; t.c.sc = (long long)nbf * rank[i];
                        pb.add(t);
                    }
                } else {
                    /* i is a leaf above j: K[m][q] += Beff[rows of n, .] G_j[q][.][n] */
                    if (!has_far(j)) continue;
                    for (int g = grp_off[i]; g < grp_off[i] + grp_cnt[i]; g++) {
                        const int n = g_y[g];
                        if (n < n0 || n >= n1) continue;
                        HTask t{};
                        t.M = g_cnt[g]; t.N = (int)S[j].size(); t.K = rank[j]; t.Z = 1;
                        beff(b, tr, t.a);
                        t.a.gr = P_row + g_start[g];
                        t.b.buf = KB_GH; t.b.off = goff[j] + (long long)(n - n0) * S[j].size() * rank[j];
                        t.b.sr = 1; t.b.sc = rank[j];
                        t.c.buf = KB_K; t.c.off = 0; t.c.gr = P_x + g_start[g]; t.c.sr = nbf;
                        t.c.gc = P_S[j]; t.c.sc = 1;
                        pb.add(t);
                    }
                }
            }
        }
        close_group();
        /* backward, inner nodes: H_c[n][q] += E_c H_p[n][q], level by level (:1253-1305) */
        for (int lv = minl; lv <= maxl - 1; lv++) {
            open_group("bwd-inner");
            for (int p : level_list(lv)) {
                if (nch[p] == 0 || !has_far(p) || sic[p].empty()) continue;
                for (int k = 0; k < nch[p]; k++) {
                    int cc = child(p, k);
                    if (!has_far(cc) || sic[cc].empty()) continue;
                    std::vector<int> m(sic[cc].size());
                    for (size_t t = 0; t < sic[cc].size(); t++) m[t] = pos_in(sic[p], sic[cc][t]);
                    HTask t{};
                    t.M = rank[cc]; t.N = nbf; t.K = rank[p]; t.Z = (int)sic[cc].size();
                    t.a.buf = KB_ARENA; t.a.off = (long long)uoff[p] + (long long)coff[cc] * rank[p];
                    t.a.sr = rank[p]; t.a.sc = 1;
                    t.b.buf = KB_GH; t.b.off = hoff[p]; t.b.sr = 1; t.b.sc = rank[p];
                    t.b.gz = pb.put(m); t.b.sz = (long long)nbf * rank[p];
                    t.c.buf = KB_GH; t.c.off = hoff[cc]; t.c.sr = 1; t.c.sc = rank[cc];
                    t.c.sz = (long long)nbf * rank[cc];
                    pb.add(t);
                }
            }
            close_group();
        }
        /* backward, leaves: K[m][q] += U_i[rows of n] H_i[n][q] */
        open_group("bwd-leaf");
        for (int li = 0; li < nl; li++) {
            const int i = h->height_nodes[li];
            if (!has_far(i)) continue;
            for (int g = grp_off[i]; g < grp_off[i] + grp_cnt[i]; g++) {
                const int n = g_y[g];
                if (n < n0 || n >= n1) continue;
                HTask t{};
                t.M = g_cnt[g]; t.N = nbf; t.K = rank[i]; t.Z = 1;
                t.a.buf = KB_ARENA; t.a.off = (long long)uoff[i]; t.a.gr = P_row + g_start[g];
                t.a.sr = rank[i]; t.a.sc = 1;
                t.b.buf = KB_GH; t.b.off = hoff[i] + (long long)pos_in(sic[i], n) * nbf * rank[i];
                t.b.sr = 1; t.b.sc = rank[i];
                t.c.buf = KB_K; t.c.off = 0; t.c.gr = P_x + g_start[g]; t.c.sr = nbf; t.c.sc = 1;
                pb.add(t);
            }
        }
        close_group();
        ks->chunks.push_back(ch);
    }

    const double t_tasks = secs();
    /* ---- tile counts and flops ---- */
    for (KChunk &ch : ks->chunks)
        for (KGroup &g : ch.groups)
            for (int t = g.t0; t < g.t0 + g.nt; t++) {
                const HTask &T = pb.tasks[t];
                flops += 2.0 * T.M * (double)T.N * T.K * T.Z;
                g.tiles += gemm_tiles<double>(T.M, T.N, T.Z);
            }
    ks->flops = flops;
    if (const char *v = std::getenv("H2G_KPLAN_VERBOSE"); v && v[0] == '1') {
        /* per phase of the first n range: tasks, tiles, flops, output elements, mean M / N*Z / K */
        const KChunk &ch = ks->chunks.front();
        for (const KGroup &g : ch.groups) {
            double fl = 0.0, outs = 0.0, sm = 0.0, snz = 0.0, sk = 0.0;
            for (int t = g.t0; t < g.t0 + g.nt; t++) {
                const HTask &T = pb.tasks[t];
                fl += 2.0 * T.M * (double)T.N * T.K * T.Z;
                outs += (double)T.M * T.N * T.Z;
                sm += T.M; snz += (double)T.N * T.Z; sk += T.K;
            }
            std::fprintf(stderr, "kplan %-10s tasks %7d tiles %8lld GFLOP %8.2f outputs(M) %8.2f mean M %6.1f NZ %8.1f K %6.1f\n",
                         g.phase, g.nt, g.tiles, fl / 1e9, outs / 1e6, sm / g.nt, snz / g.nt, sk / g.nt);
        }
        std::fprintf(stderr, "kplan ranges %zu, near GFLOP %.2f\n", ks->chunks.size(), 0.0);
    }
    ks->arena_elems = arena_elems;
    for (const KChunk &ch : ks->chunks) ks->gh_elems = std::max(ks->gh_elems, ch.gh_elems);

    ks->near_items = near_pre.back();

    const double t_count = secs();
    /* ---- bounds of every access, checked before anything is launched ---- */
    const size_t nbf2 = (size_t)nbf * nbf;
    for (const HTask &T : expand)
        if (!opnd_in_bounds(T.a, T.M, T.K, 1, fact_elems, pb.pool) || !opnd_in_bounds(T.b, T.K, T.N, 1, fact_elems, pb.pool) ||
            !opnd_in_bounds(T.c, T.M, T.N, 1, arena_elems, pb.pool)) {
            set_error("exchange plan: out-of-bounds block expansion");
            return 5;
        }
    for (const KChunk &ch : ks->chunks)
        for (const KGroup &g : ch.groups)
            for (int t = g.t0; t < g.t0 + g.nt; t++) {
                const HTask &T = pb.tasks[t];
                auto size_of = [&](int buf) {
                    return buf == KB_ARENA ? arena_elems : buf == KB_GH ? ch.gh_elems : nbf2;
                };
                if (!opnd_in_bounds(T.a, T.M, T.K, T.Z, size_of(T.a.buf), pb.pool) ||
                    !opnd_in_bounds(T.b, T.K, T.N, T.Z, size_of(T.b.buf), pb.pool) ||
                    !opnd_in_bounds(T.c, T.M, T.N, T.Z, size_of(T.c.buf), pb.pool)) {
                    set_error(std::string("exchange plan: out-of-bounds operand in phase ") + g.phase + ", task " +
                              std::to_string(t));
                    return 5;
                }
            }
    for (const NearTask &t : hnear) {
        int di = -1;
        for (int b = 0; b < h->n_D; b++)
            if ((size_t)t.off == doff[b]) { di = b; break; }
        if (di < 0 || t.e0 < 0 || t.e0 + t.ne > (int)e_row.size() || t.g0 < 0 || t.g0 + t.ng > (int)g_start.size()) {
            set_error("exchange plan: bad near-field task");
            return 5;
        }
        const int nr = h->c_D_blks[di]->nrow, ncb = h->c_D_blks[di]->ncol;
        const int er = t.trans ? ncb : nr, fr = t.trans ? nr : ncb;   /* rows of the e side, of the f side */
        for (int e = t.e0; e < t.e0 + t.ne; e++)
            if (e_row[e] >= er || e_x[e] >= nbf || e_y[e] >= nbf) { set_error("exchange plan: near row out of range"); return 5; }
        for (int g = t.g0; g < t.g0 + t.ng; g++)
            for (int f = g_start[g]; f < g_start[g] + g_cnt[g]; f++)
                if (f >= (int)e_row.size() || e_row[f] >= fr || e_x[f] >= nbf) {
                    set_error("exchange plan: near column out of range");
                    return 5;
                }
    }
    const double t_plan = secs();
    if (verbose)
        std::fprintf(stderr, "kplan (host): rows and column sets %.2f s, tasks %.2f s, tile counts %.2f s, bounds "
                     "check %.2f s\n", t_sets, t_tasks - t_sets, t_count - t_tasks, t_plan - t_count);
    if (!upload) return 0;

    /* ---- upload ---- */
    std::vector<int> bf_shell(nbf);
    for (int s = 0; s < nsh; s++)
        for (int i = sb[s]; i < sb[s + 1]; i++) bf_shell[i] = s;
    KCUDA_TRY(cudaMalloc(&ks->arena, arena_elems * sizeof(double)));
    KCUDA_TRY(cudaMemset(ks->arena, 0, arena_elems * sizeof(double)));
    for (int i = 0; i < n_node; i++) {
        const H2E_dense_mat_p U = h->U[i];
        if (U->nrow == 0 || rank[i] == 0) continue;
        KCUDA_TRY(cudaMemcpy2D(ks->arena + uoff[i], sizeof(double) * rank[i], U->data, sizeof(double) * U->ld,
                               sizeof(double) * rank[i], U->nrow, cudaMemcpyHostToDevice));
    }
    auto put_dense = [&](H2E_dense_mat_p m, size_t dst) -> int {
        if (m->ld < 0 || m->nrow == 0 || m->ncol == 0) return 0;
        KCUDA_TRY(cudaMemcpy2D(ks->arena + dst, sizeof(double) * m->ncol, m->data, sizeof(double) * m->ld,
                               sizeof(double) * m->ncol, m->nrow, cudaMemcpyHostToDevice));
        return 0;
    };
    for (int b = 0; b < h->n_B; b++) if (put_dense(h->c_B_blks[b], boff[b])) return 10;
    for (int b = 0; b < h->n_D; b++) if (put_dense(h->c_D_blks[b], doff[b])) return 10;
    const double t_arena = secs();
    if (!expand.empty()) {
        double *fact = nullptr;
        KCUDA_TRY(cudaMalloc(&fact, fact_elems * sizeof(double)));
        size_t k = 0;
        auto put_fact = [&](H2E_dense_mat_p m) -> int {
            if (m->ld >= 0 || m->nrow == 0 || m->ncol == 0) return 0;
            size_t n = (size_t)(m->nrow + m->ncol) * (-m->ld);
            if (n) KCUDA_TRY(cudaMemcpy(fact + fact_off[k], m->data, n * sizeof(double), cudaMemcpyHostToDevice));
            k++;
            return 0;
        };
        for (int b = 0; b < h->n_B; b++) if (put_fact(h->c_B_blks[b])) return 10;
        for (int b = 0; b < h->n_D; b++) if (put_fact(h->c_D_blks[b])) return 10;
        std::vector<GemmTask> et(expand.size());
        std::vector<long long> epre(1, 0);
        for (size_t t = 0; t < expand.size(); t++) {
            const HTask &T = expand[t];
            auto cv = [&](const HOpnd &o) {
                Opnd r{};
                r.p = (o.buf == KB_FACT ? fact : ks->arena) + o.off;
                r.gr = r.gc = r.gz = nullptr;
                r.sr = o.sr; r.sc = o.sc; r.sz = o.sz;
                return r;
            };
            et[t].a = cv(T.a); et[t].b = cv(T.b); et[t].c = cv(T.c);
            et[t].M = T.M; et[t].N = T.N; et[t].K = T.K; et[t].Z = 1;
            epre.push_back(epre.back() + gemm_tiles<double>(T.M, T.N, 1));
        }
        if (epre.back() > 0x7fffffffLL) { set_error("exchange: expansion launch too large"); return 4; }
        std::vector<int> etask;
        for (size_t t = 0; t < expand.size(); t++) etask.insert(etask.end(), (size_t)(epre[t + 1] - epre[t]), (int)t);
        etask.push_back(0);
        GemmTask *dtask = nullptr;
        long long *dpre = nullptr;
        int *dtt = nullptr;
        KCUDA_TRY(cudaMalloc(&dtask, et.size() * sizeof(GemmTask)));
        KCUDA_TRY(cudaMalloc(&dpre, epre.size() * sizeof(long long)));
        KCUDA_TRY(cudaMalloc(&dtt, etask.size() * sizeof(int)));
        KCUDA_TRY(cudaMemcpy(dtask, et.data(), et.size() * sizeof(GemmTask), cudaMemcpyHostToDevice));
        KCUDA_TRY(cudaMemcpy(dpre, epre.data(), epre.size() * sizeof(long long), cudaMemcpyHostToDevice));
        KCUDA_TRY(cudaMemcpy(dtt, etask.data(), etask.size() * sizeof(int), cudaMemcpyHostToDevice));
        k_gemm<double><<<(unsigned)epre.back(), kGThreads>>>(dtask, dpre, (int)et.size(), dtt);
        KCUDA_TRY(cudaGetLastError());
        KCUDA_TRY(cudaDeviceSynchronize());
        cudaFree(dtask);
        cudaFree(dpre);
        cudaFree(dtt);
        cudaFree(fact);
    }
    pb.pool.push_back(0);
    KCUDA_TRY(cudaMalloc(&ks->pool, pb.pool.size() * sizeof(int)));
    KCUDA_TRY(cudaMemcpy(ks->pool, pb.pool.data(), pb.pool.size() * sizeof(int), cudaMemcpyHostToDevice));
    KCUDA_TRY(cudaMalloc(&ks->sb, (nsh + 1) * sizeof(int)));
    KCUDA_TRY(cudaMemcpy(ks->sb, sb, (nsh + 1) * sizeof(int), cudaMemcpyHostToDevice));
    KCUDA_TRY(cudaMalloc(&ks->bf_shell, nbf * sizeof(int)));
    KCUDA_TRY(cudaMemcpy(ks->bf_shell, bf_shell.data(), nbf * sizeof(int), cudaMemcpyHostToDevice));
    KCUDA_TRY(cudaMalloc(&ks->sig, (size_t)nsh * nsh * sizeof(int)));
    KCUDA_TRY(cudaMalloc(&ks->dp, (size_t)nbf * nbf * sizeof(double)));
    KCUDA_TRY(cudaMalloc(&ks->kbuf, (size_t)nbf * nbf * sizeof(double)));
    KCUDA_TRY(cudaMalloc(&ks->gh, std::max<size_t>(ks->gh_elems, 1) * sizeof(double)));

    ks->htasks.swap(pb.tasks);
    if (upload_variant<double>(ks) != 0) return 10;
    ks->n_near = (int)hnear.size();
    ks->near_items = near_pre.back();
    hnear.emplace_back();
    KCUDA_TRY(cudaMalloc(&ks->near, hnear.size() * sizeof(NearTask)));
    KCUDA_TRY(cudaMemcpy(ks->near, hnear.data(), hnear.size() * sizeof(NearTask), cudaMemcpyHostToDevice));
    KCUDA_TRY(cudaMalloc(&ks->near_start, near_pre.size() * sizeof(long long)));
    KCUDA_TRY(cudaMemcpy(ks->near_start, near_pre.data(), near_pre.size() * sizeof(long long), cudaMemcpyHostToDevice));
    ks->ext.row = ks->pool + P_row;
    ks->ext.x = ks->pool + P_x;
    ks->ext.y = ks->pool + P_ey;
    ks->ext.gs = ks->pool + P_gs;
    ks->ext.gc = ks->pool + P_gc;
    KCUDA_TRY(cudaEventCreate(&ks->ev0));
    KCUDA_TRY(cudaEventCreate(&ks->ev1));
    if (verbose)
        std::fprintf(stderr, "kplan: index sets and tasks %.2f s, arena upload %.2f s, low-rank expansion and "
                     "task upload %.2f s (%zu tasks, %zu index entries, %.2f GB arena)\n", t_plan, t_arena - t_plan,
                     secs() - t_arena, ks->htasks.size(), pb.pool.size(), arena_elems * 8e-9);
    return 0;
}

/* ======================================================================== */
/* Launch                                                                    */
/* ======================================================================== */

template <typename T>
static int enqueue_typed(KState *ks, const double *den, cudaStream_t s)
{
    const int nbf = ks->nbf, nsh = ks->nsh;
    const KVariant &v = std::is_same<T, double>::value ? ks->v64 : ks->v32;
    T *dp = std::is_same<T, double>::value ? (T *)ks->dp : (T *)ks->dp32;
    const T *arena = std::is_same<T, double>::value ? (const T *)ks->arena : (const T *)ks->arena32;
    KCUDA_TRY(cudaMemsetAsync(ks->kbuf, 0, (size_t)nbf * nbf * sizeof(double), s));
    long long n = (long long)nsh * nsh;
    k_density_sig<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(den, nbf, nsh, ks->sb, ks->sig);
    n = (long long)nbf * nbf;
    k_density_masked<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(den, nbf, nsh, ks->bf_shell, ks->sig, dp);
    if (ks->near_items > 0)
        k_near<T><<<(unsigned)((ks->near_items + 255) / 256), 256, 0, s>>>(ks->near, ks->near_start, ks->n_near, ks->ext,
                                                                           arena, dp, nbf, ks->kbuf);
    size_t gi = 0;
    for (const KChunk &ch : ks->chunks) {
        KCUDA_TRY(cudaMemsetAsync(ks->gh, 0, ch.gh_elems * sizeof(T), s));
        for (const KGroup &g : ch.groups) {
            if (std::is_same<T, float>::value && ks->use_tc) {
                const KVariant &w = ks->vtc;
                const long long nt = w.group_tiles[gi];
                if (nt > 0 && ks->use_tc == 1)
                    k_gemm_tcp<<<(unsigned)std::min<long long>(nt, ks->n_sm), kPThreads, kPSmemLaunch, s>>>(
                        w.tasks + g.t0, w.tile_start + w.group_pre[gi], g.nt, w.tile_task + w.group_tile_off[gi],
                        ks->err_dev);
                else if (nt > 0)
                    k_gemm_tc<<<(unsigned)nt, kTcThreads, kTcSmemLaunch, s>>>(
                        w.tasks + g.t0, w.tile_start + w.group_pre[gi], g.nt, w.tile_task + w.group_tile_off[gi],
                        ks->err_dev);
            } else if (v.group_tiles[gi] > 0) {
                k_gemm<T><<<(unsigned)v.group_tiles[gi], GemmCfg<T>::NT, 0, s>>>(
                    v.tasks + g.t0, v.tile_start + v.group_pre[gi], g.nt, v.tile_task + v.group_tile_off[gi]);
            }
            gi++;
        }
    }
    return 0;
}

/* K of one density on device arrays; mixed = FP32 contractions (FP64 K). */
static int enqueue_exchange(KState *ks, const double *den, double *K, cudaStream_t s, bool timed, bool mixed)
{
    (void)cudaGetLastError();   /* a stale error of an earlier, handled runtime call is not ours */
    const int nbf = ks->nbf;
    if (mixed) {
        int rc = ensure_f32(ks);
        if (rc) return rc;
    }
    if (timed) KCUDA_TRY(cudaEventRecord(ks->ev0, s));
    int rc = mixed ? enqueue_typed<float>(ks, den, s) : enqueue_typed<double>(ks, den, s);
    if (rc) return rc;
    if (K != ks->kbuf)
        KCUDA_TRY(cudaMemcpyAsync(K, ks->kbuf, (size_t)nbf * nbf * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (timed) KCUDA_TRY(cudaEventRecord(ks->ev1, s));
    KCUDA_TRY(cudaGetLastError());
    return 0;
}

static int launches_per_build(const KState *ks)
{
    int n = 2 + (ks->near_items > 0);
    for (const KChunk &ch : ks->chunks)
        for (const KGroup &g : ch.groups) n += g.tiles > 0;
    return n;
}

static std::mutex g_kmu;

static int get_kstate(H2ERI_p h, DevRep **d, KState **out)
{
    int rc = get_rep(h, d);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_kmu);
    if ((*d)->kstate == nullptr) {
        int cur = -1;
        cudaGetDevice(&cur);
        if (cur != (*d)->device) cudaSetDevice((*d)->device);
        KState *k = new KState();
        k->err_dev = (*d)->err_flag_dev;
        (*d)->kstate = k;
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
        double cap = kWorkCap;   /* an explicit budget replaces the default cap */
        if ((*d)->k_work_bytes > 0) {
            free_b = (size_t)((*d)->k_work_bytes / 0.4);
            cap = (*d)->k_work_bytes;
        }
        rc = build_kplan(h, k, free_b, true, cap);
        if (cur != (*d)->device && cur >= 0) cudaSetDevice(cur);
        if (rc) {
            free_exchange_state(*d);
            return rc;
        }
    }
    *out = (KState *)(*d)->kstate;
    return 0;
}

}  // namespace h2g

using namespace h2g;

/* ======================================================================== */
/* C API                                                                     */
/* ======================================================================== */

extern "C" int H2ERI_build_exchange_device(H2ERI_p h2eri, const double *d_den, double *d_K, void *stream)
{
    H2gRange nvtx_range("H2ERI_build_exchange_device");
    DevRep *d;
    KState *ks;
    int rc = get_kstate(h2eri, &d, &ks);
    if (rc) return rc;
    if (d_den == nullptr || d_K == nullptr) { set_error("null density or K pointer"); return 3; }
    cudaStream_t s = stream ? (cudaStream_t)stream : d->s_main;
    return enqueue_exchange(ks, d_den, d_K, s, false, d->precision == H2ERI_GPU_MIXED);
}

extern "C" int H2ERI_build_exchange_multi(H2ERI_p h2eri, int n_den, const double *den_mats, double *K_mats)
{
    H2gRange nvtx_range("H2ERI_build_exchange_multi");
    DevRep *d;
    KState *ks;
    int rc = get_kstate(h2eri, &d, &ks);
    if (rc) return rc;
    if (n_den < 1) { set_error("n_den < 1"); return 3; }
    const size_t nn = (size_t)ks->nbf * ks->nbf, bytes = nn * sizeof(double);
    float total = 0.f;
    for (int i = 0; i < n_den; i++) {
        /* the masked-density buffer doubles as the staging copy of the input:
         * k_density_masked reads element t before it writes element t */
        KCUDA_TRY(cudaMemcpyAsync(ks->dp, den_mats + i * nn, bytes, cudaMemcpyHostToDevice, d->s_main));
        rc = enqueue_exchange(ks, ks->dp, ks->kbuf, d->s_main, true, d->precision == H2ERI_GPU_MIXED);
        if (rc) return rc;
        KCUDA_TRY(cudaMemcpyAsync(K_mats + i * nn, ks->kbuf, bytes, cudaMemcpyDeviceToHost, d->s_main));
        KCUDA_TRY(cudaStreamSynchronize(d->s_main));
        if (d->err_flag != nullptr && (*d->err_flag & kTcErrBit)) {
            *d->err_flag &= ~kTcErrBit;
            set_error("the exchange tensor-core kernel gave up waiting for its MMAs (bounded wait expired); "
                      "results are invalid");
            return 11;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ks->ev0, ks->ev1);
        total += ms;
    }
    ks->last_ms = total / n_den;
    h2eri->n_matvec += n_den;
    return 0;
}

extern "C" void H2ERI_build_exchange(H2ERI_p h2eri, const double *den_mat, double *K_mat)
{
    if (H2ERI_build_exchange_multi(h2eri, 1, den_mat, K_mat) != 0) {
        std::fprintf(stderr, "[h2eri_gb300 FATAL] H2ERI_build_exchange failed: %s\n", H2ERI_gpu_last_error());
        std::fflush(stderr);
        std::abort();
    }
}

extern "C" int H2ERI_gpu_set_exchange_memory(H2ERI_p h2eri, double bytes)
{
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_kmu);
    d->k_work_bytes = bytes > 0 ? bytes : 0.0;
    free_exchange_state(d);
    return 0;
}

extern "C" int H2ERI_exchange_plan_check(H2ERI_p h2eri, double device_bytes, double *out, int n)
{
    if (h2eri == nullptr || h2eri->U == nullptr || h2eri->c_D_blks == nullptr) {
        set_error("H2 representation not built");
        return 2;
    }
    KState ks;
    int rc = build_kplan(h2eri, &ks, (size_t)device_bytes, false);
    if (rc) return rc;
    long long tiles = 0;
    for (const KChunk &ch : ks.chunks)
        for (const KGroup &g : ch.groups) tiles += g.tiles;
    double vals[5] = {ks.flops, (double)ks.chunks.size(), (double)ks.gh_elems * sizeof(double),
                      (double)ks.near_items, (double)tiles};
    for (int i = 0; i < std::min(n, 5); i++) out[i] = vals[i];
    return 0;
}

extern "C" int H2ERI_gpu_exchange_report(H2ERI_p h2eri, double *out, int n)
{
    DevRep *d;
    KState *ks;
    int rc = get_kstate(h2eri, &d, &ks);
    if (rc) return -rc;
    double vals[7] = {ks->flops, (double)ks->last_ms, (double)ks->chunks.size(),
                      (double)ks->gh_elems * sizeof(double), (double)ks->near_items, (double)launches_per_build(ks),
                      !ks->f32_ready ? -1.0 : (double)(ks->use_tc != 0)};
    int m = std::min(n, 7);
    for (int i = 0; i < m; i++) out[i] = vals[i];
    return m;
}
