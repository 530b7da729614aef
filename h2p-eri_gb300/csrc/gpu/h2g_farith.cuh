/*
 * Float-pair arithmetic of the mixed-precision kernels.
 *
 * A value is carried as an unevaluated sum hi + lo of two floats. Products
 * of a stored matrix entry a (one float, or a float pair) with a vector
 * entry x = xh + xl are accumulated error-free on the FP32 pipe: the product
 * fl(a xh) and its exact rounding error (from an FMA) are separated, the
 * rounded product is added to the running hi part with an error-free
 * two-sum (Knuth), and every error term goes to the lo part. Only the
 * storage rounding of a remains (2^-24 relative for single floats, ~2^-48
 * for pairs).
 *
 * Blackwell executes two FP32 operations per instruction on 64-bit register
 * pairs (add/sub/mul/fma .f32x2); the pk_* helpers use them, so the
 * compensated update of two independent sums costs one issue slot per step.
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
__device__ __forceinline__ float2 pk_mul(float2 a, float2 b)
{
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
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

/* Vector entry prepared for products: (xh, xl) and -xh, each broadcast to
 * both halves of a pair. */
struct XIn {
    float2 h, nh, l;
};
__device__ __forceinline__ XIn xin(float xh, float xl)
{
    XIn r;
    r.h = bcast(xh);
    r.nh = bcast(-xh);
    r.l = bcast(xl);
    return r;
}

/* (sh, sl) += a * x for two independent sums (one per half), a single
 * floats. With np = fl(a * -xh) = -fl(a xh), e = fma(a, xh, np) is the exact
 * rounding error of the product; s = sh - np is the two-sum of sh and the
 * rounded product. 11 packed operations. */
__device__ __forceinline__ void pk_cacc1(float2 &sh, float2 &sl, float2 a, const XIn &x)
{
    const float2 np = pk_mul(a, x.nh);
    const float2 e = pk_fma(a, x.h, np);
    const float2 c = pk_fma(a, x.l, e);
    const float2 s = pk_sub(sh, np);
    const float2 bp = pk_sub(s, sh);
    const float2 t2 = pk_sub(sh, pk_sub(s, bp));
    const float2 err = pk_sub(t2, pk_add(np, bp));
    sh = s;
    sl = pk_add(sl, pk_add(err, c));
}

/* Same for float-pair entries a = ah + al (12 packed operations). */
__device__ __forceinline__ void pk_cacc2(float2 &sh, float2 &sl, float2 ah, float2 al, const XIn &x)
{
    const float2 np = pk_mul(ah, x.nh);
    const float2 e = pk_fma(ah, x.h, np);
    const float2 c = pk_fma(ah, x.l, pk_fma(al, x.h, e));
    const float2 s = pk_sub(sh, np);
    const float2 bp = pk_sub(s, sh);
    const float2 t2 = pk_sub(sh, pk_sub(s, bp));
    const float2 err = pk_sub(t2, pk_add(np, bp));
    sh = s;
    sl = pk_add(sl, pk_add(err, c));
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
