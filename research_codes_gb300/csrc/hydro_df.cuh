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
// splits of their FP64 values.  The artificial-viscosity part of the
// pressure factor and of du/dt, the signal velocities and diffu stay FP32:
// they do not cancel at that level.  The kernel constant -5 c1 common to
// every term (W1(q) = c1 u^3 (u - 1 - 4q) = -5 c1 q u^3 with u = 1 - q,
// hdr_kernel.hpp:251-257) is applied to the finished sums in FP64.
//
// The pair set is the one the signal-velocity kernel marks (every j inside
// the support of i or j, plus a few just beyond both, whose terms are
// exactly zero: u = max(1 - q, 0) = 0), without self pairs (equal ids,
// hdr_hydro.hpp:356).  That kernel writes each i-particle's marked j indices
// into a fixed-capacity row; an i-particle whose row overflowed is summed by
// one warp over its walk's whole list instead.
#pragma once

#include <vector_types.h>

#include "df32.cuh"

namespace sphk {

// FP32C hydro records of one particle (FP32C mode of hydro_kernel):
//   phi (x_hi, y_hi, z_hi, mass)      plo (x_lo, y_lo, z_lo, -)
//   vhi (vx_hi, vy_hi, vz_hi, 1/h)    vlo (vx_lo, vy_lo, vz_lo, h^-4)
//   g1  (P_hi, P_lo, presc_hi, bswt/2) g2 (dens, vsnd, alph, alphu)
//   g3  (thrm_hi, thrm_lo, eta, presc_lo)
//   g4  (1/h hi, 1/h lo, h^-4 hi, h^-4 lo)
struct HydroDFI {
    float xh, yh, zh, xl, yl, zl;
    float vxh, vyh, vzh, vxl, vyl, vzl;
    dfk::df presc, hinv, h4;
    float eta, dens, vsnd, bswt, alph, alphu, ph, pl, th, tl;
};

// Sums over j: acceleration a, softening correction g, the pressure part
// of du/dt without its factor P_i Omega_i / rho_i^2 (ud: sum ka w), the
// viscous part (uv: sum ka visc, FP32 terms) and diffu (dif).
struct HydroDFAcc {
    dfk::df ax, ay, az, gx, gy, gz, ud, uv, dif;
};

DF_HD HydroDFI hydro_df_i(float4 phi, float4 plo, float4 vhi, float4 vlo, float4 g1, float4 g2, float4 g3,
                          float4 g4) {
    HydroDFI i;
    i.xh = phi.x; i.yh = phi.y; i.zh = phi.z;
    i.xl = plo.x; i.yl = plo.y; i.zl = plo.z;
    i.vxh = vhi.x; i.vyh = vhi.y; i.vzh = vhi.z;
    i.vxl = vlo.x; i.vyl = vlo.y; i.vzl = vlo.z;
    i.presc = dfk::make(g1.z, g3.w);
    i.hinv = dfk::make(g4.x, g4.y);
    i.h4 = dfk::make(g4.z, g4.w);
    i.eta = g3.z; i.dens = g2.x; i.vsnd = g2.y; i.bswt = g1.w; i.alph = g2.z; i.alphu = g2.w;
    i.ph = g1.x; i.pl = g1.y; i.th = g3.x; i.tl = g3.y;
    return i;
}

DF_HD HydroDFAcc hydro_df_zero() {
    const dfk::df z = dfk::make(0.0f, 0.0f);
    return HydroDFAcc{z, z, z, z, z, z, z, z, z};
}

// q u^3 h^-4 with q = r / h, u = max(1 - q, 0): the kernel-gradient factor
// W1(q) h^-4 / (-5 c1) (hdr_kernel.hpp:251-257), exactly zero for q >= 1.
DF_HD dfk::df hydro_df_grad(dfk::df r, dfk::df hinv, dfk::df h4) {
    using namespace dfk;
    const df q = mul(r, hinv);
    // 1 - q.h is exact for q.h in [1/2, 2] and Fast2Sum-exact below; beyond,
    // u < 0 and the factor is zero
    const df s = fast_two_sum(1.0f, -q.h);
    const df u = fast_two_sum(s.h, sub(s.l, q.l));
    if (!(u.h > 0.0f)) return make(0.0f, 0.0f);
    return mul(mul(q, mul(sqr(u), u)), h4);
}

// One pair (i, j) of calcHydro (hdr_hydro.hpp:349-398) added to acc; j given
// by its records.  The pair must not be a self pair.
DF_HD void hydro_df_pair(const HydroDFI &i, float4 phi, float4 plo, float4 vhi, float4 vlo, float4 g1, float4 g2,
                         float4 g3, float4 g4, HydroDFAcc &acc) {
    using namespace dfk;
    const df dx = diff(i.xh, i.xl, phi.x, plo.x);
    const df dy = diff(i.yh, i.yl, phi.y, plo.y);
    const df dz = diff(i.zh, i.zl, phi.z, plo.z);
    const df r2 = add(add(sqr(dx), sqr(dy)), sqr(dz));
    const df ri = rsqrt(r2);
    const df r = mul(r2, ri);
    const df dwi = hydro_df_grad(r, i.hinv, i.h4);
    const df dwj = hydro_df_grad(r, make(g4.x, g4.y), make(g4.z, g4.w));
    const df ka = mul(add(dwi, dwj), phi.w);   // (dW_i + dW_j) m_j / (-5 c1)
    // velocity projection w = v_ij . r_ij / r, and the viscosity (FP32)
    const df ux = diff(i.vxh, i.vxl, vhi.x, vlo.x);
    const df uy = diff(i.vyh, i.vyl, vhi.y, vlo.y);
    const df uz = diff(i.vzh, i.vzl, vhi.z, vlo.z);
    const df w = mul(add(add(mul(dx, ux), mul(dy, uy)), mul(dz, uz)), ri);
    const float wneg = w.h < 0.0f ? w.h : 0.0f;
    const float vs = i.vsnd + g2.y - 3.0f * wneg;
    const float rhi = 1.0f / (i.dens + g2.x);
    const float av = (i.bswt + g1.w) * (i.alph + g2.z) * vs * wneg;
    // pressure gradient with the viscous pressure, :378-382
    const df pf = add(add(i.presc, make(g1.z, g3.w)), -0.5f * av * rhi);
    const df fa = mul(mul(pf, ka), ri);
    accumulate(acc.ax, mul(fa, dx));
    accumulate(acc.ay, mul(fa, dy));
    accumulate(acc.az, mul(fa, dz));
    // energy equation with conduction, :384-393: ka (P_i Omega_i / rho_i^2 w
    // - visc), the first part summed without its constant factor
    const float du = (i.th - g3.x) + (i.tl - g3.y);
    const float dp = (i.ph - g1.x) + (i.pl - g1.y);
    const float vsu2 = fabsf(dp) * rhi * 2.0f;
    const float vsu = vsu2 > 0.0f ? sqrtf(vsu2) : 0.0f;
    const float visc = rhi * (0.25f * av * wneg - (i.alphu + g2.w) * vsu * du);
    accumulate(acc.ud, mul(ka, w));
    accumulate(acc.uv, ka.h * visc);
    accumulate(acc.dif, rhi * du * ka.h * ri.h);
    // softening correction, :395-398
    const df dg = mul(mul(add(mul(dwi, i.eta), mul(dwj, g3.z)), ri), phi.w);
    accumulate(acc.gx, mul(dg, dx));
    accumulate(acc.gy, mul(dg, dy));
    accumulate(acc.gz, mul(dg, dz));
}

// The reference's outputs from the sums: acch = 0.5 sum(-fa dx),
// accg = 0.5 sum(dg dx), udot = 0.5 sum(...), diffu = 2 sum(...)
// (hdr_hydro.hpp:401-421), with the factor -5 c1 of every term.
DF_HD void hydro_df_finish(const HydroDFAcc &a, const HydroDFI &i, double c1, double *acch, double *accg,
                           double *udot, double *diffu) {
    const double k = -5.0 * c1;
    acch[0] = -0.5 * k * dfk::to_double(a.ax);
    acch[1] = -0.5 * k * dfk::to_double(a.ay);
    acch[2] = -0.5 * k * dfk::to_double(a.az);
    accg[0] = 0.5 * k * dfk::to_double(a.gx);
    accg[1] = 0.5 * k * dfk::to_double(a.gy);
    accg[2] = 0.5 * k * dfk::to_double(a.gz);
    *udot = 0.5 * k * (dfk::to_double(i.presc) * dfk::to_double(a.ud) - dfk::to_double(a.uv));
    *diffu = 2.0 * k * dfk::to_double(a.dif);
}

}  // namespace sphk
