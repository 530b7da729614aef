/*
 * Multi-density H2 apply on the tensor cores (tcgen05), mixed mode.
 *
 * Self-test of the operand layouts: h2g_selftest_umma multiplies one
 * 128 x 128 bf16 tile by 16 vectors on both sides, N = A X^T and
 * T = A^T Y^T, through the same shared-memory layouts and descriptors as
 * the production kernel (A K-major for N, the same bytes MN-major for T), so
 * a test can compare with exact integer arithmetic on the host.
 */
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

#include <cuda_bf16.h>

#include "h2g_gpu_api.h"
#include "h2g_umma.cuh"

namespace h2g {

constexpr int kStRows = 128, kStCols = 128, kStVec = 16;
constexpr uint32_t kStSmem = 40 * 1024;              /* A 32 KB, X 4 KB, Y 4 KB */
constexpr uint32_t kStSmemLaunch = kStSmem + 1024;   /* + slack to align the window to 1024 bytes */

__global__ void __launch_bounds__(128, 1) k_umma_selftest(const float *__restrict__ A, const float *__restrict__ X,
                                                          const float *__restrict__ Y, float *__restrict__ N,
                                                          float *__restrict__ T)
{
    extern __shared__ __align__(16) unsigned char sm_raw[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    /* 128-byte swizzle atoms must start on 1024-byte boundaries */
    unsigned char *sm = sm_raw + ((1024u - (umma::smem_u32(sm_raw) & 1023u)) & 1023u);
    unsigned char *sA = sm, *sX = sm + 32768, *sY = sm + 32768 + 4096;
    for (uint32_t i = tid * 16; i < kStSmem; i += 128 * 16) *reinterpret_cast<uint4 *>(sm + i) = make_uint4(0, 0, 0, 0);
    __syncthreads();
    for (int i = tid; i < kStRows * kStCols; i += 128) {
        const int r = i / kStCols, c = i % kStCols;
        *reinterpret_cast<__nv_bfloat16 *>(sA + umma::kmajor_off(r, c, 16384)) = __float2bfloat16_rn(A[i]);
    }
    for (int i = tid; i < kStVec * kStCols; i += 128) {
        const int v = i / kStCols, k = i % kStCols;
        *reinterpret_cast<__nv_bfloat16 *>(sX + umma::kmajor_off(v, k, 2048)) = __float2bfloat16_rn(X[i]);
        *reinterpret_cast<__nv_bfloat16 *>(sY + umma::kmajor_off(v, k, 2048)) = __float2bfloat16_rn(Y[i]);
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(umma::smem_u32(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    umma::fence_async_smem();
    if (warp == 0) umma::tmem_alloc(&tmem_base, 32);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tm = tmem_base;
    if (tid == 0) {
        const uint32_t a0 = umma::smem_u32(sA), x0 = umma::smem_u32(sX), y0 = umma::smem_u32(sY);
        const uint32_t idN = umma::idesc_bf16(128, 16, 0, 0), idT = umma::idesc_bf16(128, 16, 1, 0);
        for (int kk = 0; kk < 8; kk++) {
            const uint64_t ad = umma::sdesc(a0 + (kk / 4) * 16384 + (kk % 4) * 32, 16, 1024);
            const uint64_t bd = umma::sdesc(x0 + (kk / 4) * 2048 + (kk % 4) * 32, 16, 1024);
            umma::mma_bf16(tm, ad, bd, idN, kk > 0);
        }
        for (int kk = 0; kk < 8; kk++) {
            const uint64_t ad = umma::sdesc(a0 + kk * 2048, 16384, 1024);
            const uint64_t bd = umma::sdesc(y0 + (kk / 4) * 2048 + (kk % 4) * 32, 16, 1024);
            umma::mma_bf16(tm + 16, ad, bd, idT, kk > 0);
        }
        umma::mma_commit(umma::smem_u32(&bar));
    }
    /* bounded wait for the MMAs (about a second of SM clock); on expiry the
     * outputs are marked with NaN, the wait is repeated once (bounded) for
     * MMAs still in flight, and the TMEM is freed all the same */
    const uint32_t b = umma::smem_u32(&bar);
    auto wait_bar = [&]() {
        const long long t0 = clock64();
        uint32_t ok = 0;
        while (!ok) {
            asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                         "selp.u32 %0, 1, 0, p;\n\t}"
                         : "=r"(ok)
                         : "r"(b)
                         : "memory");
            if (!ok && clock64() - t0 > 2000000000LL) break;
        }
        return ok != 0;
    };
    const bool done = wait_bar();
    const int row = 32 * warp + lane;
    if (done) {
        umma::fence_after_sync();
        uint32_t rN[16], rT[16];
        umma::tmem_ld16(tm + ((uint32_t)(32 * warp) << 16), rN);
        umma::tmem_ld16(tm + ((uint32_t)(32 * warp) << 16) + 16, rT);
        umma::tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; j++) {
            N[row * kStVec + j] = __uint_as_float(rN[j]);
            T[row * kStVec + j] = __uint_as_float(rT[j]);
        }
    } else {
        for (int j = 0; j < 16; j++) N[row * kStVec + j] = T[row * kStVec + j] = __int_as_float(0x7fc00001);
        (void)wait_bar();
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tm, 32);
}

}  // namespace h2g

using namespace h2g;

/* Test hook (not part of the public header): A 128 x 128 row-major, X and Y
 * 16 x 128 (one vector per row), outputs N[128][16] = A X^T and
 * T[128][16] = A^T Y^T computed by tcgen05 MMAs from bf16 operands. Values
 * should be integers of at most 8 significant bits so that the bf16
 * operands are exact. Returns 0, or a CUDA error code. */
extern "C" int h2g_selftest_umma(const float *A, const float *X, const float *Y, float *N, float *T)
{
    float *dA = nullptr, *dX = nullptr, *dY = nullptr, *dN = nullptr, *dT = nullptr;
    const size_t nA = (size_t)kStRows * kStCols, nV = (size_t)kStVec * kStCols, nO = (size_t)128 * kStVec;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess && x != cudaSuccess) e = x; };
    chk(cudaMalloc(&dA, nA * 4));
    chk(cudaMalloc(&dX, nV * 4));
    chk(cudaMalloc(&dY, nV * 4));
    chk(cudaMalloc(&dN, nO * 4));
    chk(cudaMalloc(&dT, nO * 4));
    if (e == cudaSuccess) {
        chk(cudaMemcpy(dA, A, nA * 4, cudaMemcpyHostToDevice));
        chk(cudaMemcpy(dX, X, nV * 4, cudaMemcpyHostToDevice));
        chk(cudaMemcpy(dY, Y, nV * 4, cudaMemcpyHostToDevice));
        chk(cudaFuncSetAttribute(k_umma_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStSmemLaunch));
    }
    if (e == cudaSuccess) {
        k_umma_selftest<<<1, 128, kStSmemLaunch>>>(dA, dX, dY, dN, dT);
        chk(cudaGetLastError());
        chk(cudaDeviceSynchronize());
    }
    if (e == cudaSuccess) {
        chk(cudaMemcpy(N, dN, nO * 4, cudaMemcpyDeviceToHost));
        chk(cudaMemcpy(T, dT, nO * 4, cudaMemcpyDeviceToHost));
    }
    cudaFree(dA); cudaFree(dX); cudaFree(dY); cudaFree(dN); cudaFree(dT);
    if (e != cudaSuccess) {
        set_error(std::string("umma self-test: ") + cudaGetErrorString(e));
        return (int)e;
    }
    return 0;
}

namespace h2g {

/* ======================================================================== */
/* Multi-density tile kernel                                                 */
/* ======================================================================== */
/*
 * One CTA (512 threads, one per SM) runs 128 x 128 tiles of the stored
 * matrices for up to 16 densities at once on the tensor cores. Products of
 * an FP32 (or float-pair) matrix with FP64 vectors are formed exactly enough
 * for the mixed mode by integer slices (the scheme of Ozaki, Ogita, Oishi and
 * Rump, Numer. Algorithms 59, 2012):
 *   - each tile is equilibrated by power-of-two row and column scales
 *     2^e_r, 2^f_c (precomputed per tile) so that |a_rc| < 1, and a is cut
 *     into four signed 8-bit slices, a = sum_i s_i 2^-8(i+1), |s_0| <= 256,
 *     |s_i| <= 128 after that; the slices are computed once, when the mixed
 *     arenas are filled, and kept in device memory as bf16 in the exact
 *     byte image of the shared-memory operand (k_make_slices);
 *   - each density's 128 vector entries of the tile (column entries times
 *     2^f_c for the N side, row entries times 2^e_r for the T side) are
 *     scaled by a power of two 2^E to at most 1 and cut the same way into
 *     NLEV signed digits of 8 bits, per launch;
 *   - the slice products with i + j < NLEV run as bf16 MMAs (exact
 *     operands) into FP32 accumulators in tensor memory, one per level
 *     k = i + j. Every partial sum is an integer below 2^24, so the FP32
 *     accumulation is exact; the levels are combined in 64-bit integers,
 *     turned into doubles with integer operations and added to the FP64
 *     outputs with atomics.
 * What is dropped (slices beyond the fourth, digits and pairs beyond
 * level NLEV - 1) is below 2^-32 of the equilibrated tile; measured on the
 * C10H22 matvec it adds 8e-10 (NLEV 4) or 2e-10 (NLEV 5) to the 4.4e-9 of
 * the FP32 storage.
 *
 * Both products use one shared-memory copy of the slices: the tile is
 * stored K-major for N = A X (M = rows) and read MN-major as the operand of
 * T = A^T Y (M = columns).
 *
 * Warp roles, handing over through mbarriers:
 *   warp 0   copies the four slices of each tile into shared memory with
 *            bulk copies, slice i as soon as the MMAs of the previous tile
 *            that read slice i have completed (full[i] / freed[i]);
 *   warp 1   issues the MMAs, slice by slice as the copies land, into one of
 *            two tensor-memory buffers, then commits (mmadone[b]);
 *   warps 2-15 turn the densities' vector entries into digits (two
 *            shared-memory buffers, vfull[b]), every load of a tile issued
 *            before the first is used; warps 4-11 then run the epilogue of
 *            the previous tile (tensor-memory loads, tempty[b], level
 *            combination, FP64 atomics) while the next tiles are in flight.
 * Every wait is bounded (about a second); on expiry the kernel records it
 * in the error word, skips the remaining work, waits once more (bounded)
 * for copies and MMAs in flight and frees its tensor memory.
 */
constexpr int kMT = 512;                  /* threads                          */
constexpr int kMV = 16;                   /* densities per pass (MMA N)       */
constexpr int kSA = 4;                    /* slices of the stored matrix      */
constexpr int kSXMax = 5;                 /* largest number of vector digits  */
constexpr uint32_t kSliceA = 32768;       /* one 128 x 128 bf16 slice         */
constexpr uint32_t kSliceV = 4096;        /* one 16 x 128 bf16 vector slice   */
constexpr uint32_t kTmemCols = 512;
constexpr int kNWorkers = 14;             /* digit warps 2..15                */
constexpr int kEpiWarps = 8;              /* epilogue warps 4..11             */
constexpr int kPairsPerWorker = (2 * 16 + kNWorkers - 1) / kNWorkers;   /* (side, density) pairs */

struct MmaSmem {
    static constexpr uint32_t OFF_V = kSA * kSliceA;                          /* [2][side][kSXMax] slices */
    static constexpr uint32_t OFF_MU = OFF_V + 2 * 2 * kSXMax * kSliceV;      /* int [4][2][16]           */
    static constexpr uint32_t OFF_BAR = OFF_MU + 4 * 2 * kMV * 4;
    /* barriers: full[4], freed[4], vfull[2], mmadone[2], tempty[2]; TMEM slot; dead flag */
    static constexpr uint32_t BYTES = OFF_BAR + 14 * 8 + 16;
    static constexpr uint32_t LAUNCH = BYTES + 1024;
};
static_assert(MmaSmem::LAUNCH <= 227 * 1024, "shared memory of the multi-density kernel");

/* Vector digits of side (0: N, 1: T) in buffer b: K-major bf16 operands
 * whose rows are (digit j, density v) -> row 16 j + v, so that the digits
 * j = 0 .. n - 1 of all densities form one operand of 16 n rows. Byte
 * offset, relative to the vector region, of K block kb (64 entries) of
 * digit j; the 8-row swizzle atoms of consecutive digits are contiguous. */
__host__ __device__ constexpr uint32_t vslice(int b, int side, int kb, int j)
{
    return (uint32_t)(((b * 2 + side) * 2 + kb) * kSXMax + j) * (kSliceV / 2);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
/* bulk copy global -> shared (16-byte aligned, size a multiple of 16),
 * completing on an mbarrier; the slices are read once per launch, so the
 * copies are marked L2 evict-first */
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar), "l"(pol)
                 : "memory");
}

/* x * 2^s for a double given by its bits (zero stays zero; results below
 * the normal range flush to zero, far below the slices' resolution). */
__device__ __forceinline__ long long dbl_scale_bits(long long b, int s)
{
    const long long ex = (b >> 52) & 0x7ff;
    if (ex == 0) return 0;
    const long long ne = ex + s;
    if (ne <= 0) return 0;
    return b + ((long long)s << 52);
}

/* Exponent E with |x| <= 2^E for the largest magnitude (bits without sign). */
__device__ __forceinline__ int pow2_exp(unsigned long long mx)
{
    if (mx == 0) return 0;
    const int ex = (int)(mx >> 52);
    return ex - 1023 + ((mx & 0xFFFFFFFFFFFFFull) != 0 ? 1 : 0);
}

/* The SX signed 8-bit digits of x / 2^E (|x| <= 2^E), most significant
 * first: x / 2^E ~ sum_j d_j 2^-8(j+1), |d_0| <= 256, |d_j| <= 128 after
 * that, from the signed fixed-point value
 * q = round(x 2^(8 SX - E)) in 64 bits, biased by 128 in every digit below
 * the top so that the balanced digits d_j in [-128, 127] (j >= 1) are the
 * plain bytes of q + bias minus 128, and the top digit is what remains
 * above them (|d_0| <= 256). Bytes become floats through the exponent
 * field (2^23 + byte is exact), without conversion instructions. */
template <int SX>
__device__ __forceinline__ void dbl_digits(long long bits, int E, float (&d)[SX])
{
    const unsigned long long a = (unsigned long long)bits & 0x7FFFFFFFFFFFFFFFull;
    const int ex = (int)(a >> 52);
    long long q = 0;
    if (ex != 0) {
        const unsigned long long m = (a & 0xFFFFFFFFFFFFFull) | (1ull << 52);
        const int sh = 1075 + E - 8 * SX - ex;   /* >= 52 - 8 SX > 0 */
        if (sh < 64) q = (long long)((m + (1ull << (sh - 1))) >> sh);
        if (bits < 0) q = -q;
    }
    constexpr unsigned long long bias = 0x8080808080808080ull >> (8 * (9 - SX));   /* 128 in bytes 0 .. SX - 2 */
    const long long qb = q + (long long)bias;
#pragma unroll
    for (int j = 1; j < SX; j++) {
        const unsigned byte = (unsigned)(qb >> (8 * (SX - 1 - j))) & 255u;
        d[j] = __int_as_float(0x4B000000 | byte) - 8388736.0f;   /* 2^23 + 128 */
    }
    const int top = (int)(qb >> (8 * (SX - 1)));                   /* in [-256, 256] */
    d[0] = __int_as_float(0x4B000000 + (top + 256)) - 8388864.0f;  /* 2^23 + 256 */
}

/* I * 2^e2 as a double, built with integer operations (the FP64 pipe of
 * this part is narrow); the mantissa is truncated to 53 bits. */
__device__ __forceinline__ double i64_ldexp(long long I, int e2)
{
    if (I == 0) return 0.0;
    const unsigned long long a = I < 0 ? (unsigned long long)(-I) : (unsigned long long)I;
    const int msb = 63 - __clzll((long long)a);
    const unsigned long long m = msb > 52 ? a >> (msb - 52) : a << (52 - msb);
    const int ex = msb + e2 + 1023;
    if (ex <= 0) return 0.0;
    const unsigned long long b = ((unsigned long long)ex << 52) | (m & 0xFFFFFFFFFFFFFull) |
                                 (I < 0 ? 0x8000000000000000ull : 0ull);
    return __longlong_as_double((long long)b);
}

/* Round to an integer (ties to even) with two FP32 additions: valid for
 * |t| < 2^22. */
__device__ __forceinline__ float rint_small(float t)
{
    return __fadd_rn(__fadd_rn(t, 12582912.0f), -12582912.0f);
}

/* 8 columns (one density half) of NLEV level accumulators for the warp's
 * 32 TMEM lanes. */
template <int NLEV>
__device__ __forceinline__ void tmem_ld_levels(uint32_t taddr, uint32_t (&r)[NLEV][8])
{
#pragma unroll
    for (int k = 0; k < NLEV; k++)
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=r"(r[k][0]), "=r"(r[k][1]), "=r"(r[k][2]), "=r"(r[k][3]), "=r"(r[k][4]),
                       "=r"(r[k][5]), "=r"(r[k][6]), "=r"(r[k][7])
                     : "r"(taddr + (uint32_t)(k * kMV))
                     : "memory");
    umma::tmem_wait_ld();
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
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

/* The bf16 slices of every tile, in the byte image of the shared-memory
 * operand (K-major, 128-byte swizzle; rows past nr and columns past nc of
 * the copied atoms zero), made once when the mixed arenas are filled. One
 * CTA per tile; each thread takes two neighbouring columns of a row. */
__global__ void __launch_bounds__(256) k_make_slices(const TileM *__restrict__ tiles, const float *__restrict__ a32,
                                                     const float2 *__restrict__ a32x2,
                                                     const int8_t *__restrict__ scales, unsigned char *__restrict__ out)
{
    const TileM T = tiles[blockIdx.x];
    const int nb = (T.nc + 63) / 64, na = (T.nr + 7) / 8;
    unsigned char *o = out + T.s_off;
    const int8_t *sc = scales + (size_t)blockIdx.x * 256;
    for (int q = threadIdx.x; q < T.nr * 64; q += blockDim.x) {
        const int r = q >> 6, c = (q & 63) * 2;
        if (c >= T.nc) continue;
        const float rf = __int_as_float((127 - sc[r]) << 23);
        float hi[2], lo[2];
        if (T.fmt == FMT_F32X2) {
            const float4 v = *reinterpret_cast<const float4 *>(a32x2 + T.a2 + (size_t)r * T.ld2 + c);
            hi[0] = v.x; hi[1] = v.y; lo[0] = v.z; lo[1] = v.w;
        } else {
            const float2 v = *reinterpret_cast<const float2 *>(a32 + T.a2 + (size_t)r * T.ld2 + c);
            hi[0] = v.x; hi[1] = v.y; lo[0] = lo[1] = 0.f;
        }
        float s[kSA][2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const float cf = (c + u < T.nc) ? __int_as_float((127 - sc[128 + c + u]) << 23) : 0.f;
            /* scaled step by step: |hi rf| <= 1 and |hi rf cf| < 1, while rf cf
             * alone can exceed the float range for rows of tiny entries */
            float tt = hi[u] * rf * cf * 256.f;
            const float tl = lo[u] * rf * cf * 256.f;
            s[0][u] = rint_small(tt);
            tt = ((tt - s[0][u]) + tl) * 256.f;
#pragma unroll
            for (int i = 1; i < kSA; i++) {
                s[i][u] = rint_small(tt);
                tt = (tt - s[i][u]) * 256.f;
            }
        }
        const uint32_t off = (uint32_t)(r / 8) * 1024u + (uint32_t)(r % 8) * 128u +
                             (uint32_t)(((c % 64) / 8) ^ (r % 8)) * 16u + (uint32_t)(c % 8) * 2u;
#pragma unroll
        for (int i = 0; i < kSA; i++) {
            const size_t blk = ((size_t)i * nb + c / 64) * na * 1024;
            *reinterpret_cast<__nv_bfloat162 *>(o + blk + off) = __floats2bfloat162_rn(s[i][0], s[i][1]);
        }
    }
}

template <int NLEV>
__global__ void __launch_bounds__(kMT, 1)
k_tile_mma(const TileM *__restrict__ tiles, int n_tiles, const __grid_constant__ VecArgs va0, int nvec0,
           const unsigned char *__restrict__ slices, const int8_t *__restrict__ scales, unsigned *err,
           const BatchMol *__restrict__ mols)
{
    /* one structure: va0 / nvec0 and slice offsets into `slices`; a batch
     * (mols != nullptr): every tile names its structure, and its slice
     * offset is the slices' device address (slices is null) */
    auto tva = [&](const TileM &T) -> const VecArgs & { return mols ? mols[T.mol].va : va0; };
    auto tnv = [&](const TileM &T) { return min(kMV, (mols ? mols[T.mol].nvec : nvec0) - (int)blockIdx.y * kMV); };
    constexpr int SX = NLEV;                     /* vector digits */
    constexpr int TPB = 2 * NLEV * kMV;          /* TMEM columns per buffer */
    static_assert(SX <= kSXMax && 2 * TPB <= (int)kTmemCols, "layout");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *sm = smem_raw + ((1024u - (umma::smem_u32(smem_raw) & 1023u)) & 1023u);
    int *smu = reinterpret_cast<int *>(sm + MmaSmem::OFF_MU);   /* [k % 4][side][16] */
    const uint32_t sA = umma::smem_u32(sm), sV = sA + MmaSmem::OFF_V;
    const uint32_t bar0 = sA + MmaSmem::OFF_BAR;
    auto full = [&](int i) { return bar0 + 8u * i; };
    auto freed = [&](int i) { return bar0 + 32u + 8u * i; };
    auto vfull = [&](int b) { return bar0 + 64u + 8u * b; };
    auto mmadone = [&](int b) { return bar0 + 80u + 8u * b; };
    auto tempty = [&](int b) { return bar0 + 96u + 8u * b; };
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + MmaSmem::OFF_BAR + 112);
    volatile int *dead = reinterpret_cast<volatile int *>(sm + MmaSmem::OFF_BAR + 116);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int vg = blockIdx.y * kMV;
    const int nk = (n_tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;   /* tiles of this CTA */

    /* the slice buffer starts zeroed: rows and columns that a partial tile
     * does not copy keep finite values from then on */
    for (uint32_t o = (uint32_t)tid * 16; o < (uint32_t)kSA * kSliceA; o += kMT * 16)
        *reinterpret_cast<uint4 *>(sm + o) = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        for (int i = 0; i < kSA; i++) { mbar_init(full(i), 1); mbar_init(freed(i), 1); }
        for (int b = 0; b < 2; b++) {
            mbar_init(vfull(b), kNWorkers);
            mbar_init(mmadone(b), 1);
            mbar_init(tempty(b), kEpiWarps);
        }
        *dead = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    umma::fence_async_smem();
    if (warp == 0) umma::tmem_alloc(tmem_slot, kTmemCols);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    auto wait = [&](uint32_t bar, uint32_t parity) -> bool {   /* false once anything expired */
        if (*dead) return false;
        if (mbar_wait_bounded(bar, parity)) return true;
        atomicOr(err, 1u);
        *dead = 1;
        return false;
    };

    if (warp == 0) {
        /* ---------------- slice copies ---------------- */
        if (lane == 0) {
            int issued = 0;
            for (int k = 0; k < nk; k++) {
                const TileM T = tiles[blockIdx.x + k * gridDim.x];
                const int nb = (T.nc + 63) / 64, na = (T.nr + 7) / 8;
                const uint32_t chunk = (uint32_t)na * 1024u;
                bool ok = true;
                for (int i = 0; i < kSA; i++) {
                    if (k > 0 && !wait(freed(i), (uint32_t)((k - 1) & 1))) { ok = false; break; }
                    mbar_expect_tx(full(i), chunk * nb);
                    for (int b = 0; b < nb; b++)
                        bulk_g2s(sA + i * kSliceA + b * 16384,
                                 reinterpret_cast<const unsigned char *>((uintptr_t)slices + T.s_off) +
                                     ((size_t)i * nb + b) * chunk,
                                 chunk, full(i));
                }
                if (!ok) break;
                issued = k + 1;
            }
            /* after an expiry: copies still in flight land before the CTA exits */
            if (*dead && issued > 0)
                for (int i = 0; i < kSA; i++) (void)mbar_wait_bounded(full(i), (uint32_t)((issued - 1) & 1));
        }
    } else if (warp == 1) {
        /* ---------------- MMA issue ---------------- */
        if (lane == 0) {
            const uint64_t dN0 = umma::sdesc(sA, 16, 1024), dT0 = umma::sdesc(sA, 16384, 1024);
            const uint64_t dV0 = umma::sdesc(sV, 16, 1024);
            int committed = 0;
            for (int k = 0; k < nk; k++) {
                const TileM T = tiles[blockIdx.x + k * gridDim.x];
                const bool opN = T.k_out0 != VK_NONE, opT = T.k_out1 != VK_NONE;
                const int b = k & 1;
                if (!wait(vfull(b), (uint32_t)((k >> 1) & 1))) break;
                if (k >= 2 && !wait(tempty(b), (uint32_t)(((k - 2) >> 1) & 1))) break;
                umma::fence_after_sync();
                const uint32_t tb = tmem + (uint32_t)(b * TPB);
                bool ok = true;
                for (int i = 0; i < kSA; i++) {
                    if (!wait(full(i), (uint32_t)(k & 1))) { ok = false; break; }
                    umma::fence_after_sync();
                    /* slice i times the digits j = 0 .. NLEV - 1 - i of all
                     * densities in one MMA of N = 16 (NLEV - i): its columns
                     * are the accumulators of levels i .. NLEV - 1, in order.
                     * Every level is first written by slice 0 at K step 0. */
                    const uint32_t idN = umma::idesc_bf16(128, kMV * (NLEV - i), 0, 0);
                    const uint32_t idT = umma::idesc_bf16(128, kMV * (NLEV - i), 1, 0);
#pragma unroll
                    for (int kk = 0; kk < 8; kk++) {
                        const bool acc = !(i == 0 && kk == 0);
                        const uint32_t vk = (uint32_t)(kk & 3) * 32;
                        if (opN)
                            umma::mma_bf16(tb + i * kMV,
                                           dN0 + (((uint32_t)i * kSliceA + (kk >> 2) * 16384 + (kk & 3) * 32) >> 4),
                                           dV0 + ((vslice(b, 0, kk >> 2, 0) + vk) >> 4), idN, acc);
                        if (opT)
                            umma::mma_bf16(tb + (NLEV + i) * kMV, dT0 + (((uint32_t)i * kSliceA + kk * 2048) >> 4),
                                           dV0 + ((vslice(b, 1, kk >> 2, 0) + vk) >> 4), idT, acc);
                    }
                    umma::mma_commit(freed(i));   /* slice i may be reloaded once these are done */
                }
                if (!ok) break;
                umma::mma_commit(mmadone(b));
                committed = k + 1;
            }
            if (*dead && committed > 0)
                (void)mbar_wait_bounded(mmadone((committed - 1) & 1), (uint32_t)(((committed - 1) >> 1) & 1));
        }
    } else {
        /* ---------------- vector digits and epilogue ---------------- */
        const bool epi = warp >= 4 && warp < 4 + kEpiWarps;
        const int wk = warp - 2;                            /* 0 .. kNWorkers - 1 */
        const int side = (warp - 4) >> 2, q = warp & 3;    /* epilogue warps */
        const int idx = 32 * q + lane;                      /* row (N) or column (T) of the tile */
        auto epilogue = [&](int k) {
            const int t = blockIdx.x + k * gridDim.x;
            const TileM T = tiles[t];
            const int b = k & 1;
            const bool on = side == 0 ? T.k_out0 != VK_NONE : T.k_out1 != VK_NONE;
            const int e_sc = scales[(size_t)t * 256 + side * 128 + idx];
            const VecArgs &va = tva(T);
            const int nv = tnv(T);
            if (!wait(mmadone(b), (uint32_t)((k >> 1) & 1))) return;
            umma::fence_after_sync();
            const int lim = side == 0 ? T.nr : T.nc;
            uint32_t acc[2][NLEV][8];
#pragma unroll
            for (int hh = 0; hh < 2; hh++)
                tmem_ld_levels<NLEV>(tmem + (uint32_t)(b * TPB + side * NLEV * kMV + 8 * hh) + ((uint32_t)(32 * q) << 16),
                                     acc[hh]);
            umma::fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty(b));        /* the MMAs of tile k + 2 may overwrite the buffer */
            if (!on || idx >= lim) return;
            double *outb = side == 0 ? vec_ptr(va, T.k_out0, T.out0, 0) : vec_ptr(va, T.k_out1, T.out1, 0);
            const long long ostride = va.stride[side == 0 ? T.k_out0 : T.k_out1];
            const int *mu = smu + (k & 3) * 32 + side * 16;
#pragma unroll
            for (int hh = 0; hh < 2; hh++)
#pragma unroll
                for (int dd = 0; dd < 8; dd++) {
                    const int v = 8 * hh + dd;
                    if (v >= nv) break;
                    long long I = 0;
#pragma unroll
                    for (int lv = 0; lv < NLEV; lv++)
                        I += (long long)__float2int_rn(__uint_as_float(acc[hh][lv][dd])) << (8 * (NLEV - 1 - lv));
                    if (I == 0) continue;
                    atomicAdd(outb + (long long)(vg + v) * ostride + idx, i64_ldexp(I, e_sc + mu[v] - 8 * NLEV - 8));
                }
        };
        {
            const int e0 = 4 * lane;                            /* this lane's 4 entries */
            for (int k = 0; k < nk; k++) {
                const int t = blockIdx.x + k * gridDim.x;
                const TileM T = tiles[t];
                const int b = k & 1;
                const VecArgs &va = tva(T);
                const int nv = tnv(T);
                /* every entry of this warp's (side, density) pairs, scaled by
                 * the tile's exponents (N side: x_c 2^f_c; T side: y_r 2^e_r),
                 * loaded before any is used */
                long long xb[kPairsPerWorker][4];
#pragma unroll
                for (int pp = 0; pp < kPairsPerWorker; pp++) {
                    const int p = wk + pp * kNWorkers;
                    const int side = p >> 4, v = p & 15;
                    const bool on = p < 2 * kMV && (side == 0 ? T.k_out0 != VK_NONE : T.k_out1 != VK_NONE) && v < nv;
                    const int lim = side == 0 ? T.nc : T.nr;
                    const double *src = on ? (side == 0 ? vec_ptr(va, T.k_in0, T.in0, vg + v) : vec_ptr(va, T.k_in1, T.in1, vg + v))
                                           : nullptr;
                    const char4 ex = *reinterpret_cast<const char4 *>(scales + (size_t)t * 256 + (side == 0 ? 128 : 0) + e0);
                    const int exs[4] = {ex.x, ex.y, ex.z, ex.w};
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        xb[pp][u] = 0;
                        if (on && e0 + u < lim) xb[pp][u] = dbl_scale_bits(__double_as_longlong(src[e0 + u]), exs[u]);
                    }
                }
                /* the buffer is free once the MMAs of tile k - 2 that read it are done */
                if (k >= 2 && !wait(mmadone(b), (uint32_t)(((k - 2) >> 1) & 1))) break;
#pragma unroll
                for (int pp = 0; pp < kPairsPerWorker; pp++) {
                    const int p = wk + pp * kNWorkers;
                    if (p >= 2 * kMV) break;
                    const int side = p >> 4, v = p & 15;
                    if (!(side == 0 ? T.k_out0 != VK_NONE : T.k_out1 != VK_NONE)) continue;
                    unsigned long long mx = 0;
#pragma unroll
                    for (int u = 0; u < 4; u++) mx = max(mx, (unsigned long long)xb[pp][u] & 0x7FFFFFFFFFFFFFFFull);
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                    const int E = pow2_exp(mx);
                    if (lane == 0) smu[(k & 3) * 32 + side * 16 + v] = E;
                    float d[4][SX];
#pragma unroll
                    for (int u = 0; u < 4; u++) dbl_digits<SX>(xb[pp][u], E, d[u]);
                    unsigned char *dst = sm + MmaSmem::OFF_V + umma::kmajor_off(v, e0 & 63, 0);
#pragma unroll
                    for (int sl = 0; sl < SX; sl++) {
                        __nv_bfloat162 p0 = __floats2bfloat162_rn(d[0][sl], d[1][sl]);
                        __nv_bfloat162 p1 = __floats2bfloat162_rn(d[2][sl], d[3][sl]);
                        *reinterpret_cast<uint2 *>(dst + vslice(b, side, e0 >> 6, sl)) =
                            make_uint2(*reinterpret_cast<uint32_t *>(&p0), *reinterpret_cast<uint32_t *>(&p1));
                    }
                }
                umma::fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(vfull(b));
                if (epi && k >= 1) epilogue(k - 1);
                if (*dead) break;
            }
            if (epi && nk >= 1 && !*dead) epilogue(nk - 1);
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (warp == 0) umma::tmem_dealloc(tmem, kTmemCols);
}

/* Kernel attributes (dynamic shared memory above 48 KB) of every
 * instantiation; called when a structure is uploaded. */
int mma_init(DevRep *d)
{
    const int launch = (int)MmaSmem::LAUNCH;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess && x != cudaSuccess) e = x; };
    chk(cudaFuncSetAttribute(k_tile_mma<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, launch));
    chk(cudaFuncSetAttribute(k_tile_mma<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, launch));
    int sms = 0;
    chk(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d->device));
    if (e != cudaSuccess) {
        set_error(std::string("multi-density kernel set-up: ") + cudaGetErrorString(e));
        return 10;
    }
    d->n_sm = sms;
    return 0;
}

/* Pre-computed slices of every tile, made on the first use of the
 * tensor-core kernel (a launch with at least mma_min_vec densities, or the
 * autotuner trying it), after the mixed arenas and the tiles' exponents are
 * on the device: about 8 bytes per stored element, which a structure that
 * never runs several densities per launch does not hold. */
int mma_make_slices(DevRep *d)
{
    if (d->n_mtiles == 0 || d->mslices != nullptr) return 0;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess && x != cudaSuccess) e = x; };
    chk(cudaMalloc(&d->mslices, std::max<size_t>(d->mslice_bytes, 16)));
    chk(cudaMemset(d->mslices, 0, std::max<size_t>(d->mslice_bytes, 16)));
    if (e == cudaSuccess) {
        k_make_slices<<<d->n_mtiles, 256>>>(d->mtiles, d->arena32, d->arena32x2, d->mscales, d->mslices);
        chk(cudaGetLastError());
        chk(cudaDeviceSynchronize());
    }
    if (e != cudaSuccess) {
        set_error(std::string("multi-density slices: ") + cudaGetErrorString(e));
        return 10;
    }
    return 0;
}

/* One range of multi-density tiles for nvec densities (groups of 16 on the
 * grid's y dimension), persistent CTAs (one per SM at most). */
void launch_range_mma(const DevRep *d, const Range &r, const VecArgs &va, int nvec, cudaStream_t s)
{
    if (r.count <= 0) return;
    const int ctas = std::max(1, d->n_sm / std::max(1, d->cfg.mma_grid_div));
    const dim3 grid((unsigned)std::min(r.count, ctas), (unsigned)((nvec + kMV - 1) / kMV));
    const TileM *t = d->mtiles + r.first;
    const int8_t *sc = d->mscales + (size_t)r.first * 256;
    const int launch = (int)MmaSmem::LAUNCH;
    if (d->mma_levels == 4)
        k_tile_mma<4><<<grid, kMT, launch, s>>>(t, r.count, va, nvec, d->mslices, sc, d->err_flag_dev, nullptr);
    else
        k_tile_mma<5><<<grid, kMT, launch, s>>>(t, r.count, va, nvec, d->mslices, sc, d->err_flag_dev, nullptr);
}

/* One range of a batch plan (every structure with at most 16 densities). */
void launch_batch_mma(const TileM *tiles, const int8_t *scales, const BatchMol *mols, int count, int levels, int n_sm,
                      unsigned *err, cudaStream_t s)
{
    if (count <= 0) return;
    const dim3 grid((unsigned)std::min(count, std::max(n_sm, 1)), 1);
    VecArgs none;
    std::memset(&none, 0, sizeof(none));
    const int launch = (int)MmaSmem::LAUNCH;
    if (levels == 4)
        k_tile_mma<4><<<grid, kMT, launch, s>>>(tiles, count, none, 0, nullptr, scales, err, mols);
    else
        k_tile_mma<5><<<grid, kMT, launch, s>>>(tiles, count, none, 0, nullptr, scales, err, mols);
}

}  // namespace h2g
