// ff.cuh — double-float ("ff") arithmetic for the FP64-accurate polish.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi) / 2: about 48 significant bits (relative rounding ~2^-47
// per operation) over FP32's exponent range.  On this part the FP64 pipe
// runs at 1/64 of the FP32 rate, so an ff operation of 6-25 FP32
// instructions is several times cheaper than the FP64 operation it stands
// in for.  The building blocks are the published error-free
// transformations:
//   * two_sum (Knuth, TAOCP vol. 2, 4.2.2): s + e == a + b exactly;
//   * fast_two_sum (Dekker 1971, |a| >= |b|): the same with three operations;
//   * two_prod with a fused multiply-add: p + e == a * b exactly.
// Products and sums inside the transformations use the _rn intrinsics,
// which the compiler never contracts into an FMA (a contracted a*b + c
// would break the exactness the transformations rely on).
//
// Functions: reciprocal and reciprocal square root by one Newton step in ff
// from the SFU seed refined in FP32; e^x table-driven (Tang 1989: x =
// (32k + j) ln2/32 + r, |r| <= ln2/64, e^r by its Taylor series to r^6, 2^(j/32)
// from a 32-entry ff table); ln x by one Newton step on e^y = x from the SFU
// log2 seed (the step squares the seed's ~2^-22 error).  Each result is
// accurate to a few units of 2^-47 relative (ln: absolute, for arguments
// near 1).  Inputs must stay inside FP32's normal range; callers check the
// ranges of their exponents and fall back to FP64 otherwise.
#pragma once

#include <cuda_runtime.h>

// Linkage of the larger functions: out of line by default, so that the
// polish's seven model terms share one copy each instead of inlining dozens
// (the kernel is otherwise bound by instruction fetch).
#ifndef LCF_FF_BIG
#define LCF_FF_BIG static __device__ __noinline__
#endif
#ifndef LCF_FF_SMALL
#define LCF_FF_SMALL __device__ __forceinline__
#endif

namespace lcf {

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ffm(float hi, float lo) {
    ff r;
    r.hi = hi;
    r.lo = lo;
    return r;
}
__device__ __forceinline__ ff ff_from(double x) {
    float h = (float)x;
    return ffm(h, (float)(x - (double)h));
}
__device__ __forceinline__ double ff_to(ff a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ float two_sum(float a, float b, float& e) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}
__device__ __forceinline__ float fast_two_sum(float a, float b, float& e) {
    float s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
    return s;
}
__device__ __forceinline__ ff ff_norm(float s, float e) {
    float lo;
    float hi = fast_two_sum(s, e, lo);
    return ffm(hi, lo);
}

// a + b ("sloppy" sum: absolute error ~2^-47 (|a| + |b|))
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    float e;
    float s = two_sum(a.hi, b.hi, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return ff_norm(s, e);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ffm(-a.hi, -a.lo); }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_add(ff a, float b) {
    float e;
    float s = two_sum(a.hi, b, e);
    e = __fadd_rn(e, a.lo);
    return ff_norm(s, e);
}
__device__ __forceinline__ ff ff_add(float a, ff b) { return ff_add(b, a); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return ff_norm(p, e);
}
__device__ __forceinline__ ff ff_mul(ff a, float b) {
    float p = __fmul_rn(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return ff_norm(p, e);
}
__device__ __forceinline__ ff ff_mul(float a, ff b) { return ff_mul(b, a); }
// exact scaling by a power of two
__device__ __forceinline__ ff ff_scale(ff a, float p2) { return ffm(a.hi * p2, a.lo * p2); }
__device__ __forceinline__ ff ff_sqr(ff a) {
    float p = __fmul_rn(a.hi, a.hi);
    float e = fmaf(a.hi, a.hi, -p);
    e = fmaf(2.0f * a.hi, a.lo, e);
    return ff_norm(p, e);
}

__device__ __forceinline__ float sfu_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sfu_rsqrt(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sfu_lg2(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// 1 / b: FP32 Newton step on the SFU seed, then one ff step
// r = r1 + r1 (1 - b r1), the residual formed in ff.
LCF_FF_SMALL ff ff_rcp(ff b) {
    float r0 = sfu_rcp(b.hi);
    float r1 = fmaf(r0, fmaf(-b.hi, r0, 1.0f), r0);
    ff br = ff_mul(b, r1);                             // ~1
    float e = __fsub_rn(__fsub_rn(1.0f, br.hi), br.lo); // 1 - b r1 (1 - br.hi is exact)
    return ff_norm(r1, __fmul_rn(r1, e));
}
__device__ __forceinline__ ff ff_div(ff a, ff b) { return ff_mul(a, ff_rcp(b)); }

// 1 / sqrt(b): y = y1 + y1 (1 - b y1^2) / 2, the residual in ff.
LCF_FF_SMALL ff ff_rsqrt(ff b) {
    float y0 = sfu_rsqrt(b.hi);
    float y1 = y0 * fmaf(-0.5f * b.hi * y0, y0, 1.5f);
    float q = __fmul_rn(y1, y1);
    ff y2 = ffm(q, fmaf(y1, y1, -q));                 // y1^2 exactly
    ff by = ff_mul(b, y2);                             // ~1
    float e = __fsub_rn(__fsub_rn(1.0f, by.hi), by.lo);
    return ff_norm(y1, __fmul_rn(0.5f * y1, e));
}

// 2^(j/32), j = 0..31, as ff pairs.  In global memory, read through the L1:
// the lanes of a warp index it divergently, which the constant cache would
// serialise.
static __device__ const float2 g_exp2_tab[32] = {
    {1.0f, 0.0f},
    {1.0218971967697144f, -4.811559861650494e-08f},
    {1.0442737340927124f, 4.8334701574503924e-08f},
    {1.0671404600143433f, -5.9337519786595294e-08f},
    {1.0905077457427979f, -1.3077539939843064e-08f},
    {1.114386796951294f, -5.435540018083884e-08f},
    {1.1387885808944702f, 5.386222312608879e-08f},
    {1.1637248992919922f, -4.051441493402308e-08f},
    {1.1892070770263672f, 3.797635272917432e-08f},
    {1.215247392654419f, -3.267394887984665e-08f},
    {1.2418577671051025f, 4.496838101886169e-08f},
    {1.2690509557724f, 1.419333317542737e-09f},
    {1.2968395948410034f, -4.018999533172973e-08f},
    {1.3252366781234741f, -3.496373324196611e-08f},
    {1.3542555570602417f, -1.0123349269974824e-08f},
    {1.3839099407196045f, -5.875577357983275e-08f},
    {1.4142135381698608f, 2.4203234971764687e-08f},
    {1.4451807737350464f, 3.324199937537742e-08f},
    {1.4768261909484863f, -4.500898853621038e-08f},
    {1.5091644525527954f, -2.4959373234878512e-08f},
    {1.5422108173370361f, 8.070904833346049e-09f},
    {1.5759809017181396f, -5.661025426206834e-08f},
    {1.610490322113037f, 9.836217174097328e-09f},
    {1.6457555294036865f, -5.124972091152813e-08f},
    {1.6817928552627563f, -2.4755326677450284e-08f},
    {1.7186193466186523f, -4.8496175963919086e-08f},
    {1.7562521696090698f, -9.235770370707996e-09f},
    {1.7947090864181519f, -1.141504490931311e-08f},
    {1.8340080976486206f, -1.1239277952768134e-08f},
    {1.8741676807403564f, -4.663005626071026e-08f},
    {1.9152065515518188f, 9.845328108326612e-09f},
    {1.9571441411972046f, -1.7021804410433106e-08f}};

constexpr float FF_EXP_MAX = 88.0f;   // e^88 = 1.65e38 < FLT_MAX
constexpr float FF_EXP_MIN = -87.0f;  // below: flushed to 0

// e^x.  x.hi above FF_EXP_MAX is clamped there (callers keep their exponents
// below it or fall back to FP64); below FF_EXP_MIN the result is 0.
LCF_FF_BIG ff ff_exp(ff x) {
    if (x.hi < FF_EXP_MIN) return ffm(0.0f, 0.0f);
    if (x.hi > FF_EXP_MAX) x = ffm(FF_EXP_MAX, 0.0f);
    const float INV = 46.16624130844683f;        // 32 / ln 2
    // ln2 / 32 = L1 + L2 + L3, L1 with 12 significant bits: n * L1 is exact
    // for |n| < 4096 (|x| <= 88 gives |n| <= 4063)
    const float L1 = 0.02165985107421875f, L2 = 9.983182280848268e-07f, L3 = 5.14560928046269e-14f;
    // n = rint(x * 32/ln2) by the 1.5 * 2^23 shifter (|x * 32/ln2| < 2^22)
    const float sh = __fadd_rn(__fmul_rn(x.hi, INV), 12582912.0f);
    const int n = __float_as_int(sh) - 0x4B400000;
    const float nf = __fsub_rn(sh, 12582912.0f);
    const float t1 = __fsub_rn(x.hi, __fmul_rn(nf, L1));  // exact (Sterbenz)
    const float p2 = __fmul_rn(nf, L2);
    const float p2l = fmaf(nf, L2, -p2);
    float e;
    float s = two_sum(t1, -p2, e);
    e = __fadd_rn(e, __fsub_rn(__fsub_rn(x.lo, p2l), __fmul_rn(nf, L3)));
    const ff r = ff_norm(s, e);  // |r| <= ln2/64 + tiny
    // e^r - 1 = r + r^2 (1/2 + r (1/6 + r (1/24 + r (1/120 + r/720))))
    const float rh = r.hi;
    const float qt = rh * (0.041666666666666664f + rh * (0.008333333333333333f + rh * 0.001388888888888889f));
    const ff q = ff_add(ffm(0.1666666716337204f, -4.967053879312289e-09f), qt);
    const ff h = ff_add(ff_mul(r, q), 0.5f);
    const ff p = ff_add(r, ff_mul(ff_sqr(r), h));
    const float2 tj = __ldg(&g_exp2_tab[n & 31]);
    const ff T = ffm(tj.x, tj.y);
    const ff v = ff_add(T, ff_mul(T, p));
    const int k = n >> 5;  // floor(n / 32), in [-126, 126]
    return ff_scale(v, __int_as_float((k + 127) << 23));
}
__device__ __forceinline__ ff ff_exp(float x) { return ff_exp(ffm(x, 0.0f)); }

// ln x for x > 0 in FP32's normal range.
LCF_FF_BIG ff ff_log(ff x) {
    const float y0 = sfu_lg2(x.hi) * 0.6931471805599453f;
    const ff m = ff_mul(x, ff_exp(-y0));               // x e^-y0 = 1 + eps
    const ff e = ff_add(m, -1.0f);                      // exact: m ~ 1
    // y = y0 + ln(1 + eps) = y0 + eps - eps^2 / 2 (|eps| ~ 2^-22)
    float err;
    float s = two_sum(y0, e.hi, err);
    err = __fadd_rn(err, __fsub_rn(e.lo, 0.5f * e.hi * e.hi));
    return ff_norm(s, err);
}

// Ordering of double-float pairs (normalised: |lo| <= ulp(hi) / 2).
__device__ __forceinline__ bool ff_lt(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool ff_le(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }

// One dimension of a particle move (src/parametric.rs:1721-1735) in
// double-float: velocity w v0 + 1.5 r1 (pb - x0) + 1.5 r2 (g - x0) with the
// draws' products 1.5 r as pairs (a1, a2), clamped to +-vmax; the position
// clamped to the box, where the velocity becomes 0.
__device__ __forceinline__ void ff_move(ff x0, ff v0, ff pb, ff g, ff w, float2 a1, float2 a2, ff vm, ff lo, ff hi,
                                        ff& xn, ff& vn) {
    ff vv = ff_add(ff_add(ff_mul(w, v0), ff_mul(ffm(a1.x, a1.y), ff_sub(pb, x0))), ff_mul(ffm(a2.x, a2.y), ff_sub(g, x0)));
    if (ff_lt(vv, ff_neg(vm))) vv = ff_neg(vm);
    if (ff_lt(vm, vv)) vv = vm;
    const ff nx = ff_add(x0, vv);
    if (ff_le(nx, lo)) { xn = lo; vn = ffm(0.0f, 0.0f); }
    else if (ff_le(hi, nx)) { xn = hi; vn = ffm(0.0f, 0.0f); }
    else { xn = nx; vn = vv; }
}

}  // namespace lcf
