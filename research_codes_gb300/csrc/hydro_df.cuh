// hydro_df.cuh — the cancelling sums of calcHydro (hdr_hydro.hpp:349-398)
// in double-float arithmetic, for the FP32C engine.
//
// Near hydrostatic equilibrium the SPH pressure gradient of a particle is a
// sum of ~50 pair terms whose typical size is ~R/h times the sum (up to
// ~10^3 times at a star's centre, where the acceleration vanishes).  Every
// FP32 rounding inside a term — the separation, 1/r, q = r/h, u = 1 - q, the
// (1 - q)^3 factor, P Omega / rho^2, h^-4 — then shows up multiplied by that
// ratio, so FP32 terms reach 1e-4 relative error on such particles.  Here
// the three sums that cancel (acceleration, softening correction, du/dt) are
// formed with double-float operands and accumulators (~44 bits, df32.cuh):
// separations from the hi/lo particle records, 1/r by one Newton step,
// q and u in double-float, P Omega / rho^2 and h^-1, h^-4 from double-float
// splits of their FP64 values, the masses as hi/lo pairs (an FP32 mass
// alone would scale every term of a star's equal-mass particles by the same
// rounding, ~4e-8).  The artificial-viscosity part of the
// pressure factor and of du/dt, the signal velocities and diffu stay FP32:
// they do not cancel at that level.  The kernel constant -5 c1 common to
// every term (W1(q) = c1 u^3 (u - 1 - 4q) = -5 c1 q u^3 with u = 1 - q,
// hdr_kernel.hpp:251-257) is applied to the finished sums in FP64.
//
// The pair formula is written once over a lane type T (df32.cuh): float for
// one pair at a time, pk for two pairs of the same i-particle in the two
// halves of packed f32x2 instructions.  It uses the lean (unnormalised)
// double-float operations: ~2^-44 relative error per term, far below the
// ~10^-9 that a condition number of 10^3 and a 10^-5 target leave.
//
// The pair set is the one the signal-velocity kernel marks (every j inside
// the support of i or j, plus a few just beyond both, whose terms are
// exactly zero: u = max(1 - q, 0) = 0), without self pairs (equal ids,
// hdr_hydro.hpp:356).  That kernel writes each i-particle's marked j indices
// into a fixed-capacity row; an i-particle whose row overflowed is summed by
// one block over its walk's whole list instead.
#pragma once

#include <vector_types.h>

#include "df32.cuh"

namespace sphk {

// FP32C hydro records of one particle (FP32C mode of hydro_kernel):
//   phi (x_hi, y_hi, z_hi, mass_hi)   plo (x_lo, y_lo, z_lo, mass_lo)
//   vhi (vx_hi, vy_hi, vz_hi, 1/h)    vlo (vx_lo, vy_lo, vz_lo, h^-4)
//   g1  (P_hi, P_lo, presc_hi, bswt/2) g2 (dens, vsnd, alph, alphu)
//   g3  (thrm_hi, thrm_lo, eta, presc_lo)
//   g4  (1/h hi, 1/h lo, h^-4 hi, h^-4 lo)
// as the fields the pair formula reads, over lane type T.
template <class T>
struct HydroDFP {
    T xh, yh, zh, xl, yl, zl;
    dfk::dv<T> m;
    T vxh, vyh, vzh, vxl, vyl, vzl;
    dfk::dv<T> presc, hinv, h4;
    T eta, dens, vsnd, bswt, alph, alphu, ph, pl, th, tl;
};

DF_HD HydroDFP<float> hydro_df_rec(float4 phi, float4 plo, float4 vhi, float4 vlo, float4 g1, float4 g2, float4 g3,
                                   float4 g4) {
    HydroDFP<float> p;
    p.xh = phi.x; p.yh = phi.y; p.zh = phi.z; p.m = dfk::dv<float>{phi.w, plo.w};
    p.xl = plo.x; p.yl = plo.y; p.zl = plo.z;
    p.vxh = vhi.x; p.vyh = vhi.y; p.vzh = vhi.z;
    p.vxl = vlo.x; p.vyl = vlo.y; p.vzl = vlo.z;
    p.presc = dfk::dv<float>{g1.z, g3.w};
    p.hinv = dfk::dv<float>{g4.x, g4.y};
    p.h4 = dfk::dv<float>{g4.z, g4.w};
    p.eta = g3.z; p.dens = g2.x; p.vsnd = g2.y; p.bswt = g1.w; p.alph = g2.z; p.alphu = g2.w;
    p.ph = g1.x; p.pl = g1.y; p.th = g3.x; p.tl = g3.y;
    return p;
}

// Sums over j: acceleration a, softening correction g, the pressure part
// of du/dt without its factor P_i Omega_i / rho_i^2 (ud: sum ka w), the
// viscous part (uv: sum ka visc, FP32 terms) and diffu (dif).
template <class T>
struct HydroDFAcc {
    dfk::dv<T> ax, ay, az, gx, gy, gz, ud, uv, dif;
};

template <class T>
DF_HD HydroDFAcc<T> hydro_df_zero() {
    const dfk::dv<T> z{dfk::cst<T>(0.0f), dfk::cst<T>(0.0f)};
    return HydroDFAcc<T>{z, z, z, z, z, z, z, z, z};
}

// Per-lane operations that have no packed instruction.
DF_HD float lane_min0(float x) { return x < 0.0f ? x : 0.0f; }
DF_HD float lane_rcp(float x) { return 1.0f / x; }
DF_HD float lane_sqrt0(float x) { return x > 0.0f ? sqrtf(x) : 0.0f; }
DF_HD float lane_abs(float x) { return fabsf(x); }
// u, or exactly zero where u.h <= 0 (beyond the support)
DF_HD dfk::dv<float> lane_pos(dfk::dv<float> u) {
    return (u.h > 0.0f) ? u : dfk::dv<float>{0.0f, 0.0f};
}
DF_HD dfk::pk lane_min0(dfk::pk x) {
    const float2 v = dfk::unpack(x);
    return dfk::pack(lane_min0(v.x), lane_min0(v.y));
}
DF_HD dfk::pk lane_rcp(dfk::pk x) {
    const float2 v = dfk::unpack(x);
    return dfk::pack(1.0f / v.x, 1.0f / v.y);
}
DF_HD dfk::pk lane_sqrt0(dfk::pk x) {
    const float2 v = dfk::unpack(x);
    return dfk::pack(lane_sqrt0(v.x), lane_sqrt0(v.y));
}
DF_HD dfk::pk lane_abs(dfk::pk x) {
    dfk::pk r;
    r.v = x.v & 0x7fffffff7fffffffull;
    return r;
}
DF_HD dfk::dv<dfk::pk> lane_pos(dfk::dv<dfk::pk> u) {
    const float2 h = dfk::unpack(u.h), l = dfk::unpack(u.l);
    const bool a = h.x > 0.0f, b = h.y > 0.0f;
    return dfk::dv<dfk::pk>{dfk::pack(a ? h.x : 0.0f, b ? h.y : 0.0f), dfk::pack(a ? l.x : 0.0f, b ? l.y : 0.0f)};
}
// two particles' records in the two lanes, and one particle's in both
DF_HD dfk::dv<dfk::pk> pack_dv(dfk::dv<float> a, dfk::dv<float> b) {
    return dfk::dv<dfk::pk>{dfk::pack(a.h, b.h), dfk::pack(a.l, b.l)};
}
DF_HD HydroDFP<dfk::pk> hydro_df_pack(const HydroDFP<float> &a, const HydroDFP<float> &b) {
    using dfk::pack;
    HydroDFP<dfk::pk> p;
    p.xh = pack(a.xh, b.xh); p.yh = pack(a.yh, b.yh); p.zh = pack(a.zh, b.zh);
    p.xl = pack(a.xl, b.xl); p.yl = pack(a.yl, b.yl); p.zl = pack(a.zl, b.zl);
    p.m = pack_dv(a.m, b.m);
    p.vxh = pack(a.vxh, b.vxh); p.vyh = pack(a.vyh, b.vyh); p.vzh = pack(a.vzh, b.vzh);
    p.vxl = pack(a.vxl, b.vxl); p.vyl = pack(a.vyl, b.vyl); p.vzl = pack(a.vzl, b.vzl);
    p.presc = pack_dv(a.presc, b.presc);
    p.hinv = pack_dv(a.hinv, b.hinv);
    p.h4 = pack_dv(a.h4, b.h4);
    p.eta = pack(a.eta, b.eta); p.dens = pack(a.dens, b.dens); p.vsnd = pack(a.vsnd, b.vsnd);
    p.bswt = pack(a.bswt, b.bswt); p.alph = pack(a.alph, b.alph); p.alphu = pack(a.alphu, b.alphu);
    p.ph = pack(a.ph, b.ph); p.pl = pack(a.pl, b.pl); p.th = pack(a.th, b.th); p.tl = pack(a.tl, b.tl);
    return p;
}
// lane 0 and lane 1 of a packed double-float
DF_HD dfk::df lane0(dfk::dv<dfk::pk> x) {
    return dfk::df{dfk::unpack(x.h).x, dfk::unpack(x.l).x};
}
DF_HD dfk::df lane1(dfk::dv<dfk::pk> x) {
    return dfk::df{dfk::unpack(x.h).y, dfk::unpack(x.l).y};
}

// q u^3 h^-4 with q = r / h, u = max(1 - q, 0): the kernel-gradient factor
// W1(q) h^-4 / (-5 c1) (hdr_kernel.hpp:251-257), exactly zero for q >= 1.
template <class T>
DF_HD dfk::dv<T> hydro_df_grad(dfk::dv<T> r, dfk::dv<T> hinv, dfk::dv<T> h4) {
    using namespace dfk;
    const dv<T> q = mul_t(r, hinv);
    // u = 1 - q: Fast2Sum of 1 and -q.h (its error term exact for q.h <= 1;
    // beyond, u <= 0 and the factor is zero), then q's lo part
    const T one = cst<T>(1.0f);
    const T uh = sub(one, q.h);
    const dv<T> u = lane_pos(dv<T>{uh, sub(sub(sub(one, uh), q.h), q.l)});
    return mul_t(mul_t(q, mul_t(sqr_t(u), u)), h4);
}

// One pair (i, j) of calcHydro (hdr_hydro.hpp:349-398) added to acc.  The
// pair must not be a self pair.
template <class T>
DF_HD void hydro_df_pair(const HydroDFP<T> &i, const HydroDFP<T> &j, HydroDFAcc<T> &acc) {
    using namespace dfk;
    const dv<T> dx = diff_t(i.xh, i.xl, j.xh, j.xl);
    const dv<T> dy = diff_t(i.yh, i.yl, j.yh, j.yl);
    const dv<T> dz = diff_t(i.zh, i.zl, j.zh, j.zl);
    const dv<T> r2 = add_t(add_t(sqr_t(dx), sqr_t(dy)), sqr_t(dz));
    const dv<T> ri = rsqrt_t(r2);
    const dv<T> r = mul_t(r2, ri);
    const dv<T> dwi = hydro_df_grad(r, i.hinv, i.h4);
    const dv<T> dwj = hydro_df_grad(r, j.hinv, j.h4);
    const dv<T> ka = mul_t(add_t(dwi, dwj), j.m);   // (dW_i + dW_j) m_j / (-5 c1)
    // velocity projection w = v_ij . r_ij / r, and the viscosity (FP32)
    const dv<T> ux = diff_t(i.vxh, i.vxl, j.vxh, j.vxl);
    const dv<T> uy = diff_t(i.vyh, i.vyl, j.vyh, j.vyl);
    const dv<T> uz = diff_t(i.vzh, i.vzl, j.vzh, j.vzl);
    const dv<T> w = mul_t(add_t(add_t(mul_t(dx, ux), mul_t(dy, uy)), mul_t(dz, uz)), ri);
    // FP32 values of the unnormalised w, ka and 1/r for the FP32 terms (h
    // alone may be a few ulps off)
    const T wneg = lane_min0(add(w.h, w.l));
    const T vs = dfk::fma(cst<T>(-3.0f), wneg, add(i.vsnd, j.vsnd));
    const T rhi = lane_rcp(add(i.dens, j.dens));
    const T av = mul(mul(mul(add(i.bswt, j.bswt), add(i.alph, j.alph)), vs), wneg);
    // pressure gradient with the viscous pressure, :378-382
    const dv<T> pf = add_t(add_t(i.presc, j.presc), mul(mul(cst<T>(-0.5f), av), rhi));
    const dv<T> fa = mul_t(mul_t(pf, ka), ri);
    accumulate_t(acc.ax, mul_t(fa, dx));
    accumulate_t(acc.ay, mul_t(fa, dy));
    accumulate_t(acc.az, mul_t(fa, dz));
    // energy equation with conduction, :384-393: ka (P_i Omega_i / rho_i^2 w
    // - visc), the first part summed without its constant factor
    const T du = add(sub(i.th, j.th), sub(i.tl, j.tl));
    const T dp = add(sub(i.ph, j.ph), sub(i.pl, j.pl));
    const T vsu = lane_sqrt0(mul(mul(lane_abs(dp), rhi), cst<T>(2.0f)));
    const T xneg = mul(mul(add(i.alphu, j.alphu), vsu), cst<T>(-1.0f));
    const T visc = mul(rhi, dfk::fma(xneg, du, mul(mul(cst<T>(0.25f), av), wneg)));
    accumulate_t(acc.ud, mul_t(ka, w));
    accumulate_t(acc.uv, mul_t(ka, visc));
    accumulate_t(acc.dif, mul(mul(mul(rhi, du), add(ka.h, ka.l)), add(ri.h, ri.l)));
    // softening correction, :395-398
    const dv<T> dg = mul_t(mul_t(add_t(mul_t(dwi, i.eta), mul_t(dwj, j.eta)), ri), j.m);
    accumulate_t(acc.gx, mul_t(dg, dx));
    accumulate_t(acc.gy, mul_t(dg, dy));
    accumulate_t(acc.gz, mul_t(dg, dz));
}

// The reference's outputs from the sums: acch = 0.5 sum(-fa dx),
// accg = 0.5 sum(dg dx), udot = 0.5 sum(...), diffu = 2 sum(...)
// (hdr_hydro.hpp:401-421), with the factor -5 c1 of every term.
DF_HD void hydro_df_finish(const HydroDFAcc<float> &a, dfk::dv<float> presc, double c1, double *acch,
                           double *accg, double *udot, double *diffu) {
    auto dbl = [](dfk::dv<float> x) { return (double)x.h + (double)x.l; };
    const double k = -5.0 * c1;
    acch[0] = -0.5 * k * dbl(a.ax);
    acch[1] = -0.5 * k * dbl(a.ay);
    acch[2] = -0.5 * k * dbl(a.az);
    accg[0] = 0.5 * k * dbl(a.gx);
    accg[1] = 0.5 * k * dbl(a.gy);
    accg[2] = 0.5 * k * dbl(a.gz);
    *udot = 0.5 * k * (dbl(presc) * dbl(a.ud) - dbl(a.uv));
    *diffu = 2.0 * k * dbl(a.dif);
}

}  // namespace sphk
