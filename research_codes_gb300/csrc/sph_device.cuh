// sph_device.cuh — device helpers shared by the pair kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

// 32-byte aligned FP64 quadruple (one 256-bit load on sm_103a).
typedef double4_32a dbl4;
__host__ __device__ __forceinline__ dbl4 make_dbl4(double x, double y, double z, double w) {
    return make_double4_32a(x, y, z, w);
}

namespace sphk {

// Wendland C2 (3-D) constants of the reference, hdr_kernel.hpp:218-227.
constexpr double KSRH = 1.936492;
constexpr double CEFF0 = 3.342253804929802286e+00;
constexpr double CEFF1 = 1.336901521971920914e+01;

constexpr unsigned FULL = 0xffffffffu;

// A unit of work for the persistent pair kernels: up to 32 consecutive
// i-particles of one walk (i-group), processed by one warp against the walk's
// whole j-list.  x = walk, y = index of the first i-particle in the i arrays,
// z = number of i-particles (1..32), w = cost estimate (pairs) for ordering.
typedef int4 WorkItem;

template <bool F64>
struct Real;
template <>
struct Real<false> {
    typedef float T;
    typedef float2 T2;
    typedef float4 T4;
    __device__ static __forceinline__ float2 make2(float a, float b) { return make_float2(a, b); }
    __device__ static __forceinline__ float4 make4(float a, float b, float c, float d) {
        return make_float4(a, b, c, d);
    }
};
template <>
struct Real<true> {
    typedef double T;
    typedef double2 T2;
    typedef dbl4 T4;
    __device__ static __forceinline__ double2 make2(double a, double b) { return make_double2(a, b); }
    __device__ static __forceinline__ dbl4 make4(double a, double b, double c, double d) {
        return make_dbl4(a, b, c, d);
    }
};

// 1/sqrt in the working precision.  FP32 uses the hardware approximation
// rsqrt.approx.ftz.f32 (relative error ~2^-23; subnormal arguments, which
// squared distances in code units never are, flush to zero and give +inf
// like an exact 0); FP64 the library's double rsqrt.
__device__ __forceinline__ float rsqrt_r(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ double rsqrt_r(double x) { return rsqrt(x); }

// 1/x: FP32 via rcp.approx.ftz.f32 (relative error <= 2^-23), FP64 exact.
__device__ __forceinline__ float rcp_r(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ double rcp_r(double x) { return 1.0 / x; }

// q = sqrt(r2 * hinv2): FP32 by sqrt.approx (relative error ~2^-23,
// exact 0 at r2 = 0), FP64 by the library sqrt.
__device__ __forceinline__ float sqrt_q(float r2, float hinv2) {
    float q;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(q) : "f"(r2 * hinv2));
    return q;
}
__device__ __forceinline__ double sqrt_q(double r2, double hinv2) { return sqrt(r2 * hinv2); }

// sqrt for bounds that carry a relative margin far above 2^-22: FP32 by
// sqrt.approx.ftz.f32, FP64 by the library sqrt.
__device__ __forceinline__ float sqrt_bound(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ double sqrt_bound(double x) { return sqrt(x); }

// Radial kernel-gradient factor W1(q)/c1 with u = (1-q)_+ (hdr_kernel.hpp:251-257).
// The reference's form u^4 - u^3 (1+4q) subtracts two nearly equal terms for
// small q; FP32 evaluates the algebraically identical -5 q u^3 instead (no
// cancellation), FP64 keeps the reference's form.
__device__ __forceinline__ float w1_term(float q, float u, float u2, float u3, float p14) {
    (void)u; (void)u2; (void)p14;
    return -5.0f * q * u3;
}
__device__ __forceinline__ double w1_term(double q, double u, double u2, double u3, double p14) {
    (void)q; (void)u;
    return u2 * u2 - u3 * p14;
}

__device__ __forceinline__ float max0(float x) { return fmaxf(x, 0.0f); }
__device__ __forceinline__ double max0(double x) { return fmax(x, 0.0); }

// Compensated accumulator.  In FP32 mode a warp lane sums the pairs of one
// 32-wide j-tile in plain FP32 and folds the tile's partial sum into a Kahan
// pair (s, c); in FP64 mode it is a plain FP64 sum.
template <bool F64>
struct Acc;
template <>
struct Acc<false> {
    float s, c;
    __device__ __forceinline__ Acc() : s(0.0f), c(0.0f) {}
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};
template <>
struct Acc<true> {
    double s;
    __device__ __forceinline__ Acc() : s(0.0) {}
    __device__ __forceinline__ void add(double v) { s += v; }
    __device__ __forceinline__ double value() const { return s; }
};

// Sum / max over the `tpi` consecutive lanes that share one i-particle
// (tpi is a power of two <= 32; every lane of the warp must call it).
__device__ __forceinline__ double seg_sum(double v, int tpi) {
    for (int o = tpi >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}
__device__ __forceinline__ long long seg_sum(long long v, int tpi) {
    for (int o = tpi >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}
__device__ __forceinline__ double seg_max(double v, int tpi) {
    for (int o = tpi >> 1; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

// Lanes per i-particle for a work item of n_i i-particles: the largest power
// of two with n_i * tpi <= 32.
__device__ __forceinline__ int lanes_per_i(int n_i) {
    int tpi = 1;
    while (tpi < 32 && 2 * tpi * n_i <= 32) tpi <<= 1;
    return tpi;
}

__device__ __forceinline__ int ilog2_pow2(int x) { return __ffs(x) - 1; }

// Two FP32 values in one 64-bit register pair, for the packed f32x2
// arithmetic of sm_100 and later: one instruction applies the operation to
// both halves, each rounded exactly as the scalar instruction would.
struct f2 {
    unsigned long long v;
};
__device__ __forceinline__ f2 f2_make(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 f2_get(f2 x) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(x.v));
    return r;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
// a * b + c
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
// two consecutive floats of shared memory (8-byte aligned address)
__device__ __forceinline__ f2 f2_lds(const float *p) {
    f2 r;
    r.v = *reinterpret_cast<const unsigned long long *>(p);
    return r;
}

// Minimum / maximum over the 32 lanes of a warp (NaN lanes are ignored).
__device__ __forceinline__ float warp_min(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

// Bit mask of the lanes below this one.
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Axis-aligned box of a work item's i-particles, in the item's frame.
template <typename R>
struct IBox {
    R xl, yl, zl, xh, yh, zh;
    __device__ __forceinline__ void from_lanes(R x, R y, R z) {
        xl = warp_min(x); yl = warp_min(y); zl = warp_min(z);
        xh = warp_max(x); yh = warp_max(y); zh = warp_max(z);
    }
    // squared distance from (x, y, z) to the box (0 inside)
    __device__ __forceinline__ R d2(R x, R y, R z) const {
        const R dx = max0(fmax(xl - x, x - xh));
        const R dy = max0(fmax(yl - y, y - yh));
        const R dz = max0(fmax(zl - z, z - zh));
        return dx * dx + dy * dy + dz * dz;
    }
};

// Squared support radius beyond which no i-particle of the item interacts
// with a j-particle, from the lanes' h: (max h)^2 widened by 2e-4 so that the
// FP32 rounding of the pair distance cannot turn a kept pair into a dropped
// one.  Any lane with an h that is not a non-negative number makes the radius
// infinite (nothing is dropped, the pair arithmetic decides as without it).
template <typename R>
__device__ __forceinline__ R support2(double h) {
    const bool bad = __any_sync(FULL, !(h >= 0.0));
    const R hm = warp_max((R)h);
    return bad ? (R)INFINITY : hm * hm * (R)1.0002;
}

}  // namespace sphk
