/*
 * Float-pair arithmetic of the mixed-precision kernels.
 *
 * A value is carried as an unevaluated sum hi + lo of two floats. Products
 * of a stored matrix entry a (one float, or a float pair) with a vector
 * entry x = xh + xl are accumulated on the FP32 pipe to about 2^-44 of the
 * sum of their magnitudes, by anchored accumulation (below); partial sums are
 * then combined with error-free two-sums (Knuth). Only the storage rounding
 * of a matters (2^-24 relative for single floats, ~2^-48 for pairs).
 *
 * Blackwell executes two FP32 operations per instruction on 64-bit register
 * pairs (add/sub/mul/fma .f32x2); the pk_* helpers use them, so the update
 * of two independent sums costs one issue slot per step.
 * All helpers round to nearest explicitly, so the compiler cannot contract
 * the two-sum into FMAs.
 */
#ifndef H2G_FARITH_CUH
#define H2G_FARITH_CUH

#include <cuda_runtime.h>

namespace h2g {

/* ---- packed FP32 x 2 (sm_100 family) ---- */
__device__ __forceinline__ float2 pk_add(float2 a, float2 b)
{
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 pk_sub(float2 a, float2 b)
{
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 pk_fma(float2 a, float2 b, float2 c)
{
    float2 d;
    asm("{.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
__device__ __forceinline__ float2 bcast(float v) { return make_float2(v, v); }

__device__ __forceinline__ float2 pk_abs(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }

/* ---- anchored accumulation ----
 * A chain of products a_i * (xh_i + xl_i) whose high parts obey
 * sum |a_i xh_i| <= B is accumulated onto an anchor s0 = 1.5 * 2^k with
 * 2^k > 4B. The running value s then stays in [1.25, 1.75] * 2^k, a single
 * binade, so after s' = fma(a, xh, s) the part of the product that s' kept is
 * exactly s' - s, and the part it dropped, a xh - (s' - s) (at most half an
 * ulp of s), comes from a second FMA with one rounding of its own. The
 * dropped parts and the small products a * xl go to a plain float sum l; the
 * chain's value is (s - s0) + l, with s - s0 exact. This is five FP32
 * operations per product where the two-sum update (error-free product, Knuth
 * two-sum) takes eleven. The error is of order n 2^-46 B for n products
 * (n^2 2^-46 B at worst), so the anchor is only as good as the bound: B is
 * the computed sum |a_i| |xh_i| of the chain itself (one FMA per product),
 * which keeps the error within a few 1e-13 of sum |a_i x_i| even when the
 * magnitudes of a and x spread over four decades (a max|a| max|x| bound
 * loses three more digits there). */

/* The anchor 1.5 * 2^k for a chain bound b: 2^k > 4b, 2^-63 <= 2^k <= 2^123. */
__device__ __forceinline__ float anchor_of(float b)
{
    const unsigned e = (__float_as_uint(b) >> 23) & 0xffu;   /* b < 2^(e - 126) */
    const unsigned ek = min(max(e + 3u, 64u), 250u);
    return __uint_as_float((ek << 23) | 0x400000u);
}
__device__ __forceinline__ float2 anchor2(float2 b) { return make_float2(anchor_of(b.x), anchor_of(b.y)); }

/* (s, l1 + l2) += a * (xh + xl) for two independent anchored chains (one
 * per half), a single floats: 5 packed operations. The low part is kept as
 * two sums (dropped parts, small products) so that every running sum takes
 * one dependent operation per product. */
__device__ __forceinline__ void pk_aacc1(float2 &s, float2 &l1, float2 &l2, float2 a, float2 xh, float2 xl)
{
    const float2 s1 = pk_fma(a, xh, s);
    l1 = pk_add(l1, pk_fma(a, xh, pk_sub(s, s1)));
    l2 = pk_fma(a, xl, l2);
    s = s1;
}

/* Same for float-pair entries a = ah + al: 6 packed operations (the al * xl
 * term, below 2^-48 of the product, is left out). */
__device__ __forceinline__ void pk_aacc2(float2 &s, float2 &l1, float2 &l2, float2 ah, float2 al, float2 xh,
                                         float2 xl)
{
    const float2 s1 = pk_fma(ah, xh, s);
    l1 = pk_add(l1, pk_fma(al, xh, pk_fma(ah, xh, pk_sub(s, s1))));
    l2 = pk_fma(ah, xl, l2);
    s = s1;
}

/* Float-pair addition (ah + al) += (bh + bl) with an error-free two-sum on
 * the high parts; the result is left unnormalised. */
__device__ __forceinline__ void dfadd(float &ah, float &al, float bh, float bl)
{
    const float s = __fadd_rn(ah, bh);
    const float bp = __fsub_rn(s, ah);
    const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bp)), __fsub_rn(bh, bp));
    ah = s;
    al = __fadd_rn(__fadd_rn(al, bl), err);
}

/* Two float-pair additions at once (halves independent). */
__device__ __forceinline__ void pk_dfadd(float2 &ah, float2 &al, float2 bh, float2 bl)
{
    const float2 s = pk_add(ah, bh);
    const float2 bp = pk_sub(s, ah);
    const float2 err = pk_add(pk_sub(ah, pk_sub(s, bp)), pk_sub(bh, bp));
    ah = s;
    al = pk_add(pk_add(al, bl), err);
}

/* double -> float pair without FP64 arithmetic: hi keeps the sign, the
 * exponent and the leading 24 significant bits of x (truncated), lo is the
 * remaining 29 bits of the significand rounded to a float and scaled by a
 * power of two, so |x - (hi + lo)| <= 2^-47 |x|. Magnitudes below 2^-126
 * (hi) or 2^-74 (lo) are flushed to zero; no value here comes near either. */
__device__ __forceinline__ void split(double x, float &hi, float &lo)
{
    const unsigned bh = (unsigned)__double2hiint(x), bl = (unsigned)__double2loint(x);
    const unsigned sign = bh & 0x80000000u;
    const int e = (int)((bh >> 20) & 0x7ffu);     /* biased double exponent */
    const int fe = e - 896;                        /* biased float exponent of hi */
    const bool ok = fe >= 1 && fe <= 254;
    hi = __uint_as_float(ok ? (sign | ((unsigned)fe << 23) | ((bh & 0xfffffu) << 3) | (bl >> 29)) : sign);
    const int le = e - 948;                        /* biased float exponent of 2^(e - 1075) */
    const float m = __uint2float_rn(bl & 0x1fffffffu);
    const float l = (ok && le >= 1) ? m * __uint_as_float((unsigned)le << 23) : 0.0f;
    lo = __uint_as_float(__float_as_uint(l) | sign);
}

/* Exact float -> double by integer operations (keeps the conversion off the
 * FP64 pipe, which is narrow on this part): the exponent is rebiased by
 * 1023 - 127 and the mantissa moved up by 29 bits. Zeros map to zero; the
 * sub-normal floats (|f| < 2^-126) are flushed to zero, an absolute change
 * below 1.2e-38. */
__device__ __forceinline__ double f2d_exact(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned a = u & 0x7fffffffu;
    const bool normal = a >= 0x00800000u;
    const unsigned hi = (normal ? ((a >> 3) + 0x38000000u) : 0u) | (u & 0x80000000u);
    const unsigned lo = normal ? (u << 29) : 0u;
    return __hiloint2double((int)hi, (int)lo);
}

/* Add the float pair (h, l) to a double in global memory (two FP64
 * atomics, no FP64 arithmetic on the SM). */
__device__ __forceinline__ void atomic_add_pair(double *p, float h, float l)
{
    atomicAdd(p, f2d_exact(h));
    if (l != 0.0f) atomicAdd(p, f2d_exact(l));
}

}  // namespace h2g

#endif
