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

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace dfk {

struct df {
    float h, l;
};

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

}  // namespace dfk
