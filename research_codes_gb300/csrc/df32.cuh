// df32.cuh — double-float arithmetic: a value is the unevaluated sum hi + lo
// of two FP32 numbers (|lo| <= ulp(hi) / 2 once normalised), ~44 significant
// bits.  Used where FP32 pair terms cancel: the SPH pressure gradient, the
// gravitational-softening correction and du/dt of a star near hydrostatic
// equilibrium are sums of terms up to ~10^3 times larger than the sum itself,
// so one FP32 rounding per term (6e-8) would reach 1e-4 of the result.
//
// Building blocks (published error-free transformations):
//   two_sum      Knuth's TwoSum, s + e = a + b exactly (6 additions);
//   fast_two_sum Dekker's Fast2Sum, the same for |a| >= |b| (3 additions);
//   two_prod     the FMA-based TwoProduct, p + e = a * b exactly.
// The compositions are Dekker's double-length addition and multiplication
// (T. J. Dekker, "A floating-point technique for extending the available
// precision", Numer. Math. 18, 1971), with the FMA taking the place of his
// splitting.  Every operation is spelled with round-to-nearest intrinsics so
// that the compiler can neither contract nor reassociate it.
//
// The same header compiles for the host (plain C++, built without FP
// contraction), where the tests run the identical operation sequence.
#pragma once

#include <cmath>
#include <cstring>

#include <vector_types.h>

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace dfk {

// hi + lo over a lane type T (float; on the device also pk, below)
template <class T>
struct dv {
    T h, l;
};
using df = dv<float>;

DF_HD float add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
DF_HD float sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
DF_HD float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
DF_HD float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

DF_HD df make(float h, float l = 0.0f) { return df{h, l}; }

// Knuth TwoSum: s = fl(a + b), e = (a + b) - s exactly.
DF_HD df two_sum(float a, float b) {
    const float s = add(a, b);
    const float bb = sub(s, a);
    const float e = add(sub(a, sub(s, bb)), sub(b, bb));
    return df{s, e};
}
// Dekker Fast2Sum, valid for |a| >= |b| (or a == 0).
DF_HD df fast_two_sum(float a, float b) {
    const float s = add(a, b);
    return df{s, sub(b, sub(s, a))};
}
// FMA TwoProduct: p = fl(a b), e = a b - p exactly.
DF_HD df two_prod(float a, float b) {
    const float p = mul(a, b);
    return df{p, fma(a, b, -p)};
}

DF_HD df add(df x, df y) {
    const df s = two_sum(x.h, y.h);
    return fast_two_sum(s.h, add(s.l, add(x.l, y.l)));
}
DF_HD df add(df x, float b) {
    const df s = two_sum(x.h, b);
    return fast_two_sum(s.h, add(s.l, x.l));
}
DF_HD df neg(df x) { return df{-x.h, -x.l}; }
DF_HD df mul(df x, df y) {
    const float p = mul(x.h, y.h);
    float e = fma(x.h, y.h, -p);
    e = fma(x.h, y.l, e);
    e = fma(x.l, y.h, e);
    return fast_two_sum(p, e);
}
DF_HD df mul(df x, float b) {
    const float p = mul(x.h, b);
    float e = fma(x.h, b, -p);
    e = fma(x.l, b, e);
    return fast_two_sum(p, e);
}
DF_HD df sqr(df x) {
    const float p = mul(x.h, x.h);
    float e = fma(x.h, x.h, -p);
    e = fma(add(x.h, x.h), x.l, e);
    return fast_two_sum(p, e);
}
// Accumulation s += x: TwoSum of the hi parts, the rounding error and x's lo
// part gathered in s.l without renormalising (an accumulator's lo part only
// collects small terms; to_double adds it at the end).
DF_HD void accumulate(df &s, df x) {
    const df t = two_sum(s.h, x.h);
    s.l = add(s.l, add(t.l, x.l));
    s.h = t.h;
}
DF_HD void accumulate(df &s, float x) {
    const df t = two_sum(s.h, x);
    s.l = add(s.l, t.l);
    s.h = t.h;
}

// (ah + al) - (bh + bl) for two double-float splits of FP64 values (the hi
// difference is not exact in general: different signs or magnitudes).
DF_HD df diff(float ah, float al, float bh, float bl) {
    const df s = two_sum(ah, -bh);
    return fast_two_sum(s.h, add(s.l, sub(al, bl)));
}

// Approximate 1/sqrt(x) (relative error ~2^-22): the hardware MUFU on the
// device, the correctly rounded quotient on the host.
DF_HD float rsqrt_seed(float x) {
#if defined(__CUDA_ARCH__)
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return 1.0f / std::sqrt(x);
#endif
}

// 1/sqrt(x) for x > 0 to ~2^-43: one Newton-Raphson step on the seed y with
// the residual e = 1 - x y^2 formed exactly (TwoProduct for y^2, FMAs for
// x y^2; 1 - m is exact for m in [1/2, 2]), then
// 1/sqrt(x) = y (1 + e/2 + 3 e^2/8 + O(e^3)).
DF_HD df rsqrt(df x) {
    const float y = rsqrt_seed(x.h);
    const df t = two_prod(y, y);
    const float m = mul(x.h, t.h);
    float me = fma(x.h, t.h, -m);
    me = fma(x.h, t.l, me);
    me = fma(x.l, t.h, me);
    const float e = sub(sub(1.0f, m), me);
    const float c = mul(mul(e, y), fma(0.375f, e, 0.5f));
    return fast_two_sum(y, c);
}

// Nearest FP64 value (for the final, once-per-particle conversions).
DF_HD double to_double(df x) { return (double)x.h + (double)x.l; }

// hi / lo split of an FP64 value.
DF_HD df split(double v) {
    const float h = (float)v;
    return df{h, (float)(v - (double)h)};
}

// ---------------------------------------------------------------------------
// Lean double-float operations, generic over the lane type T: float, or on
// the device pk, two FP32 lanes in one 64-bit register pair that the packed
// f32x2 instructions of sm_100 and later process at once (each half rounded
// exactly as the scalar instruction would round it).  Two independent
// double-float computations then share every instruction.
//
// The results are left unnormalised: the closing Fast2Sum of Dekker's
// operations is dropped, so |l| may reach a few ulps of h instead of half
// an ulp (the operands must themselves have |l| << |h|; diff_t, whose lo
// inputs may carry the whole difference, normalises).  Every error-free transformation is kept (TwoSum of the hi parts,
// the FMA product error), so the relative error stays ~2^-44, while a
// multiplication costs 4 operations instead of 7 and an addition 8 instead
// of 11.  Callers that need a normalised value (shuffles, the final sums)
// use the operations above.

DF_HD float fms(float a, float b, float c) {   // a b - c, one rounding
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, -c);
#else
    return std::fma(a, b, -c);
#endif
}
template <class T>
DF_HD T cst(float c);
template <>
DF_HD float cst<float>(float c) { return c; }

// Packed operations: the f32x2 instructions on the device; the host
// versions apply the scalar operation per half (same results).
struct pk {
    unsigned long long v;
};
DF_HD pk pack(float a, float b) {
    pk r;
#if defined(__CUDA_ARCH__)
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
#else
    unsigned int ua, ub;
    memcpy(&ua, &a, 4);
    memcpy(&ub, &b, 4);
    r.v = (unsigned long long)ua | ((unsigned long long)ub << 32);
#endif
    return r;
}
DF_HD float2 unpack(pk x) {
    float2 r;
#if defined(__CUDA_ARCH__)
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(x.v));
#else
    const unsigned int ua = (unsigned int)x.v, ub = (unsigned int)(x.v >> 32);
    memcpy(&r.x, &ua, 4);
    memcpy(&r.y, &ub, 4);
#endif
    return r;
}
template <>
DF_HD pk cst<pk>(float c) { return pack(c, c); }
#if defined(__CUDA_ARCH__)
#define DF_PK2(name, op)                                                        \
    DF_HD pk name(pk a, pk b) {                                                 \
        pk r;                                                                   \
        asm(op ".rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));     \
        return r;                                                               \
    }
DF_PK2(add, "add")
DF_PK2(sub, "sub")
DF_PK2(mul, "mul")
#undef DF_PK2
DF_HD pk fma(pk a, pk b, pk c) {
    pk r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
#else
DF_HD pk add(pk a, pk b) {
    const float2 x = unpack(a), y = unpack(b);
    return pack(add(x.x, y.x), add(x.y, y.y));
}
DF_HD pk sub(pk a, pk b) {
    const float2 x = unpack(a), y = unpack(b);
    return pack(sub(x.x, y.x), sub(x.y, y.y));
}
DF_HD pk mul(pk a, pk b) {
    const float2 x = unpack(a), y = unpack(b);
    return pack(mul(x.x, y.x), mul(x.y, y.y));
}
DF_HD pk fma(pk a, pk b, pk c) {
    const float2 x = unpack(a), y = unpack(b), z = unpack(c);
    return pack(fma(x.x, y.x, z.x), fma(x.y, y.y, z.y));
}
#endif
DF_HD pk fms(pk a, pk b, pk c) {   // a b - c: the sign bits of c flipped
    pk nc;
    nc.v = c.v ^ 0x8000000080000000ull;
    return fma(a, b, nc);
}

// Knuth TwoSum and TwoDiff (s + e = a +- b exactly).
template <class T>
DF_HD dv<T> two_sum_t(T a, T b) {
    const T s = add(a, b);
    const T bb = sub(s, a);
    return dv<T>{s, add(sub(a, sub(s, bb)), sub(b, bb))};
}
template <class T>
DF_HD dv<T> two_diff_t(T a, T b) {
    const T s = sub(a, b);
    const T bb = sub(s, a);
    return dv<T>{s, sub(sub(a, sub(s, bb)), add(b, bb))};
}
template <class T>
DF_HD dv<T> add_t(dv<T> x, dv<T> y) {
    const dv<T> s = two_sum_t(x.h, y.h);
    return dv<T>{s.h, add(s.l, add(x.l, y.l))};
}
template <class T>
DF_HD dv<T> add_t(dv<T> x, T b) {
    const dv<T> s = two_sum_t(x.h, b);
    return dv<T>{s.h, add(s.l, x.l)};
}
template <class T>
DF_HD dv<T> mul_t(dv<T> x, dv<T> y) {
    const T p = mul(x.h, y.h);
    return dv<T>{p, fma(x.l, y.h, fma(x.h, y.l, fms(x.h, y.h, p)))};
}
template <class T>
DF_HD dv<T> mul_t(dv<T> x, T b) {
    const T p = mul(x.h, b);
    return dv<T>{p, fma(x.l, b, fms(x.h, b, p))};
}
template <class T>
DF_HD dv<T> sqr_t(dv<T> x) {
    const T p = mul(x.h, x.h);
    return dv<T>{p, fma(add(x.h, x.h), x.l, fms(x.h, x.h, p))};
}
// (ah + al) - (bh + bl) for hi/lo splits of two FP64 values, normalised
// (Fast2Sum): when the hi parts are equal or nearly so (close particles far
// from the origin) the lo difference is the whole result, not a correction.
template <class T>
DF_HD dv<T> diff_t(T ah, T al, T bh, T bl) {
    const dv<T> s = two_diff_t(ah, bh);
    const T l = add(s.l, sub(al, bl));
    const T h = add(s.h, l);
    return dv<T>{h, sub(l, sub(h, s.h))};
}
// s += x (the hi parts by TwoSum, the rest gathered in s.l)
template <class T>
DF_HD void accumulate_t(dv<T> &s, dv<T> x) {
    const dv<T> t = two_sum_t(s.h, x.h);
    s.l = add(s.l, add(t.l, x.l));
    s.h = t.h;
}
template <class T>
DF_HD void accumulate_t(dv<T> &s, T x) {
    const dv<T> t = two_sum_t(s.h, x);
    s.l = add(s.l, t.l);
    s.h = t.h;
}
DF_HD float rsqrt_seed_t(float x) { return rsqrt_seed(x); }
DF_HD pk rsqrt_seed_t(pk x) {
    const float2 v = unpack(x);
    return pack(rsqrt_seed(v.x), rsqrt_seed(v.y));
}
// 1/sqrt(x), x > 0: the Newton step of rsqrt above, its result left as the
// pair (seed, correction)
template <class T>
DF_HD dv<T> rsqrt_t(dv<T> x) {
    const T y = rsqrt_seed_t(x.h);
    const T th = mul(y, y);
    const T tl = fms(y, y, th);
    const T m = mul(x.h, th);
    const T me = fma(x.l, th, fma(x.h, tl, fms(x.h, th, m)));
    const T e = sub(sub(cst<T>(1.0f), m), me);
    return dv<T>{y, mul(mul(e, y), fma(cst<T>(0.375f), e, cst<T>(0.5f)))};
}

}  // namespace dfk
