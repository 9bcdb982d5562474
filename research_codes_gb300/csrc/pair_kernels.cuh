// pair_kernels.cuh — the three SPH pair-interaction kernels.
//
// Design (shared by density, hydro and gravity):
//  * Particle data live in HBM as FP64 structure-of-arrays (dbl4 packs).
//  * Work is a list of WorkItems (<= 32 i-particles of one walk).  A
//    persistent grid of warps pulls items from a global queue counter
//    (atomicAdd), largest items first, so walks with very different
//    neighbour counts balance across the 152 SMs.
//  * A warp streams its walk's j-list through a private 32-entry shared-memory
//    tile: lane k loads entry t+k (gathered through j_idx when the list is an
//    index list), converts it and stores it; every lane then reads the tile by
//    broadcast.  With n_i < 32 several lanes share one i-particle (tpi lanes,
//    strided over the tile) and are combined with warp shuffles.
//  * FP32C mode (F64 == false): positions and velocities are taken relative to
//    the first i-particle of the item in FP64 and rounded to FP32 at staging,
//    so pair arithmetic sees small, well-conditioned differences; each lane's
//    per-tile FP32 partial sums are folded into Kahan accumulators; the
//    per-particle tail (h update, Omega, normalisation) runs in FP64.
//  * FP64 mode (F64 == true): the same kernels in plain FP64 on global
//    coordinates, no compensation: the "plain FP64 GPU" comparator.
#pragma once

#include "sph_device.cuh"

namespace sphk {

// ---------------------------------------------------------------- density
struct DensityArgs {
    // i-particles
    const dbl4 *i_pm;    // x, y, z, mass
    const dbl4 *i_vel;   // vx, vy, vz, -
    const long long *i_id;
    const double *i_ksr;    // first guess of h (DensityEPI::ksr)
    const double *i_rs;     // search radius (DensityEPI::rs)
    // j-particles
    const dbl4 *j_pm;
    const dbl4 *j_vel;
    const long long *j_id;
    // work
    const WorkItem *items;
    int n_items;
    const int *n_items_dev; // when set, the item count is read from device memory
    const int *j_off;       // per walk: [j_off[w], j_off[w+1]) in j index space
    const int *j_idx;       // null: entries are j indices themselves
    int *queue;             // item counter, 0 at launch
    // outputs, indexed like the i arrays
    double *o_dens, *o_divv, *o_rotv, *o_grdh, *o_ksr;
    long long *o_np;
    unsigned char *o_itr;
    double eta_ksrh;        // eta * ksrh
    double ksr_max;         // clamp of h (+inf disables)
    const double *ksr_max_dev;  // when set, the clamp is read from device memory
};

template <bool F64, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
density_kernel(const DensityArgs a) {
    typedef typename Real<F64>::T R;
    typedef typename Real<F64>::T4 R4;
    __shared__ R4 s_p[WARPS][32];
    __shared__ R4 s_v[WARPS][32];
    __shared__ typename Real<F64>::T2 s_vl[WARPS][32];
    __shared__ long long s_id[WARPS][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int n_items = a.n_items_dev ? *a.n_items_dev : a.n_items;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.queue, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= n_items) return;
        const WorkItem it = a.items[item];
        const int jb = a.j_off[it.x];
        const int nj = a.j_off[it.x + 1] - jb;
        const int tpi = lanes_per_i(it.z);
        const int sh = ilog2_pow2(tpi);
        const int li = lane >> sh;
        const int sub = lane & (tpi - 1);
        const bool act = li < it.z;
        const int ii = it.y + (act ? li : 0);

        double cx = 0.0, cy = 0.0, cz = 0.0, cvx = 0.0, cvy = 0.0, cvz = 0.0;
        if (!F64) {
            const dbl4 c = a.i_pm[it.y];
            const dbl4 v = a.i_vel[it.y];
            cx = c.x; cy = c.y; cz = c.z;
            cvx = v.x; cvy = v.y; cvz = v.z;
        }
        const dbl4 pi = a.i_pm[ii];
        const dbl4 vi = a.i_vel[ii];
        const R xi = (R)(pi.x - cx), yi = (R)(pi.y - cy), zi = (R)(pi.z - cz);
        // velocities as hi + lo pairs so that dv keeps FP32 relative accuracy
        // even when the item's centre belongs to another stream
        const R vxi = (R)(vi.x - cvx), vyi = (R)(vi.y - cvy), vzi = (R)(vi.z - cvz);
        const R lxi = (R)((vi.x - cvx) - (double)vxi), lyi = (R)((vi.y - cvy) - (double)vyi),
                lzi = (R)((vi.z - cvz) - (double)vzi);
        const long long idi = a.i_id[ii];
        const double rs_i = a.i_rs[ii];
        const double ksr_max = a.ksr_max_dev ? *a.ksr_max_dev : a.ksr_max;
        double h = a.i_ksr[ii];
        double rho = 0.0;
        long long np = 0;
        bool itr = false;

        // three fixed-point passes, hdr_density.hpp:264-302
        for (int pass = 0; pass < 3; ++pass) {
            const double hinv_d = 1.0 / h;
            const R hinv = (R)hinv_d;
            Acc<F64> acc;
            int cnt = 0;
            for (int t = 0; t < nj; t += 32) {
                const int jk = t + lane;
                if (jk < nj) {
                    const int j = a.j_idx ? a.j_idx[jb + jk] : jb + jk;
                    const dbl4 p = a.j_pm[j];
                    s_p[wid][lane] = Real<F64>::make4((R)(p.x - cx), (R)(p.y - cy),
                                                      (R)(p.z - cz), (R)p.w);
                }
                __syncwarp();
                const int n = min(32, nj - t);
                R part = 0;
                for (int k = sub; k < n; k += tpi) {
                    const R4 pj = s_p[wid][k];
                    const R dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
                    const R r2 = dx * dx + dy * dy + dz * dz;
                    const R q = r2 * rsqrt_r(r2 > (R)0 ? r2 : (R)1e-30) * hinv;
                    const R u = max0((R)1 - q);
                    const R u2 = u * u;
                    part += pj.w * (u2 * u2 * ((R)1 + (R)4 * q));
                    cnt += (q < (R)1) ? 1 : 0;
                }
                acc.add(part);
                __syncwarp();
            }
            const double sum = seg_sum(acc.value(), tpi);
            const long long c = seg_sum((long long)cnt, tpi);
            rho = CEFF0 * hinv_d * hinv_d * hinv_d * sum;
            double hn = a.eta_ksrh * cbrt(pi.w / rho);
            hn = (hn < ksr_max) ? hn : ksr_max;
            np = c;
            itr = hn > rs_i;
            h = hn;
        }

        // gradient pass with the final h, hdr_density.hpp:304-349
        {
            const double hinv_d = 1.0 / h;
            const R hinv = (R)hinv_d;
            Acc<F64> g_acc, d_acc, rx_acc, ry_acc, rz_acc;
            for (int t = 0; t < nj; t += 32) {
                const int jk = t + lane;
                if (jk < nj) {
                    const int j = a.j_idx ? a.j_idx[jb + jk] : jb + jk;
                    const dbl4 p = a.j_pm[j];
                    const dbl4 v = a.j_vel[j];
                    s_p[wid][lane] = Real<F64>::make4((R)(p.x - cx), (R)(p.y - cy),
                                                      (R)(p.z - cz), (R)p.w);
                    const R hx = (R)(v.x - cvx), hy = (R)(v.y - cvy), hz = (R)(v.z - cvz);
                    s_v[wid][lane] = Real<F64>::make4(hx, hy, hz, (R)((v.x - cvx) - (double)hx));
                    s_vl[wid][lane] = Real<F64>::make2((R)((v.y - cvy) - (double)hy),
                                                       (R)((v.z - cvz) - (double)hz));
                    s_id[wid][lane] = a.j_id[j];
                }
                __syncwarp();
                const int n = min(32, nj - t);
                R pg = 0, pd = 0, prx = 0, pry = 0, prz = 0;
                for (int k = sub; k < n; k += tpi) {
                    const R4 pj = s_p[wid][k];
                    const R4 vj = s_v[wid][k];
                    const R dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
                    R ux = vxi - vj.x, uy = vyi - vj.y, uz = vzi - vj.z;
                    if (!F64) {
                        const typename Real<F64>::T2 vl = s_vl[wid][k];
                        ux += lxi - vj.w;
                        uy += lyi - vl.x;
                        uz += lzi - vl.y;
                    }
                    const R r2 = dx * dx + dy * dy + dz * dz;
                    const R ri = (idi != s_id[wid][k]) ? rsqrt_r(r2) : (R)0;
                    const R q = r2 * ri * hinv;
                    const R u = max0((R)1 - q);
                    const R u2 = u * u;
                    const R u3 = u2 * u;
                    const R p14 = (R)1 + (R)4 * q;
                    const R w0 = u2 * u2 * p14;            // W0 / c0
                    const R w1 = u2 * u2 - u3 * p14;       // W1 / c1
                    pg += pj.w * ((R)(3.0 * CEFF0) * w0 + (R)CEFF1 * q * w1);
                    const R dw = pj.w * w1 * ri;
                    pd += (ux * dx + uy * dy + uz * dz) * dw;
                    prx += (uy * dz - uz * dy) * dw;
                    pry += (uz * dx - ux * dz) * dw;
                    prz += (ux * dy - uy * dx) * dw;
                }
                g_acc.add(pg);
                d_acc.add(pd);
                rx_acc.add(prx);
                ry_acc.add(pry);
                rz_acc.add(prz);
                __syncwarp();
            }
            const double hinv4 = hinv_d * hinv_d * hinv_d * hinv_d;
            const double grdh = -hinv4 * seg_sum(g_acc.value(), tpi);
            const double divv = -CEFF1 * hinv4 * seg_sum(d_acc.value(), tpi);
            const double rx = CEFF1 * hinv4 * seg_sum(rx_acc.value(), tpi);
            const double ry = CEFF1 * hinv4 * seg_sum(ry_acc.value(), tpi);
            const double rz = CEFF1 * hinv4 * seg_sum(rz_acc.value(), tpi);
            if (act && sub == 0) {
                const double rhoinv = 1.0 / rho;
                const double omega = 1.0 / (1.0 + h * rhoinv * grdh / 3.0);
                const double rot2 = rx * rx + ry * ry + rz * rz;
                const double rot = (rot2 != 0.0) ? sqrt(rot2) : 0.0;
                a.o_dens[ii] = rho;
                a.o_divv[ii] = divv * rhoinv * omega;
                a.o_rotv[ii] = rot * rhoinv * omega;
                a.o_grdh[ii] = omega;
                a.o_ksr[ii] = h;
                a.o_np[ii] = np;
                a.o_itr[ii] = itr ? 1 : 0;
            }
        }
    }
}

// ---------------------------------------------------------------- hydro
struct HydroArgs {
    // i-particles (HydroEPI fields)
    const dbl4 *i_pm;    // x, y, z, (mass unused)
    const dbl4 *i_vel;
    const long long *i_id;
    const dbl4 *i_h1;    // hinv, pres, presc, bswt
    const dbl4 *i_h2;    // dens, vsnd, alph, alphu
    const double2 *i_h3;    // thrm, eta
    // j-particles (HydroEPJ fields)
    const dbl4 *j_pm;    // x, y, z, mass
    const dbl4 *j_vel;
    const long long *j_id;
    const dbl4 *j_h1;
    const dbl4 *j_h2;
    const double2 *j_h3;
    const WorkItem *items;
    int n_items;
    const int *n_items_dev;
    const int *j_off;
    const int *j_idx;
    int *queue;
    // outputs
    double *o_acch;         // 3 per particle
    double *o_accg;         // 3 per particle
    double *o_udot, *o_vsmx, *o_diffu;
};

template <bool F64, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
hydro_kernel(const HydroArgs a) {
    typedef typename Real<F64>::T R;
    typedef typename Real<F64>::T4 R4;
    __shared__ R4 s_a[WARPS][32];   // dx, dy, dz, mass
    __shared__ R4 s_b[WARPS][32];   // dvx, dvy, dvz, hinv
    __shared__ R4 s_c[WARPS][32];   // pres - pres_c, presc, bswt, dens
    __shared__ R4 s_d[WARPS][32];   // vsnd, alph, alphu, thrm - thrm_c
    __shared__ R4 s_e[WARPS][32];   // eta, hinv^4, dvx lo, dvy lo
    __shared__ R s_f[WARPS][32];    // dvz lo
    __shared__ long long s_id[WARPS][32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int n_items = a.n_items_dev ? *a.n_items_dev : a.n_items;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.queue, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= n_items) return;
        const WorkItem it = a.items[item];
        const int jb = a.j_off[it.x];
        const int nj = a.j_off[it.x + 1] - jb;
        const int tpi = lanes_per_i(it.z);
        const int sh = ilog2_pow2(tpi);
        const int li = lane >> sh;
        const int sub = lane & (tpi - 1);
        const bool act = li < it.z;
        const int ii = it.y + (act ? li : 0);

        // centre of the item: position, velocity, pressure, thermal energy
        double cx = 0, cy = 0, cz = 0, cvx = 0, cvy = 0, cvz = 0, cp = 0, cu = 0;
        if (!F64) {
            const dbl4 c = a.i_pm[it.y];
            const dbl4 v = a.i_vel[it.y];
            cx = c.x; cy = c.y; cz = c.z;
            cvx = v.x; cvy = v.y; cvz = v.z;
            cp = a.i_h1[it.y].y;
            cu = a.i_h3[it.y].x;
        }
        const dbl4 pi = a.i_pm[ii];
        const dbl4 vi = a.i_vel[ii];
        const dbl4 h1 = a.i_h1[ii];
        const dbl4 h2 = a.i_h2[ii];
        const double2 h3 = a.i_h3[ii];
        const long long idi = a.i_id[ii];
        const R xi = (R)(pi.x - cx), yi = (R)(pi.y - cy), zi = (R)(pi.z - cz);
        const R vxi = (R)(vi.x - cvx), vyi = (R)(vi.y - cvy), vzi = (R)(vi.z - cvz);
        const R lxi = (R)((vi.x - cvx) - (double)vxi), lyi = (R)((vi.y - cvy) - (double)vyi),
                lzi = (R)((vi.z - cvz) - (double)vzi);
        const R hi_i = (R)h1.x;
        const double hinv4_d = h1.x * h1.x * h1.x * h1.x;
        const R hi4_i = (R)hinv4_d;
        const R pp_i = (R)(h1.y - cp), pc_i = (R)h1.z, bs_i = (R)h1.w;
        const R dn_i = (R)h2.x, cs_i = (R)h2.y, al_i = (R)h2.z, au_i = (R)h2.w;
        const R eg_i = (R)(h3.x - cu), et_i = (R)h3.y;

        Acc<F64> ax, ay, az, ud, df, gx, gy, gz;
        R vsmx = 0;
        for (int t = 0; t < nj; t += 32) {
            const int jk = t + lane;
            if (jk < nj) {
                const int j = a.j_idx ? a.j_idx[jb + jk] : jb + jk;
                const dbl4 p = a.j_pm[j];
                const dbl4 v = a.j_vel[j];
                const dbl4 g1 = a.j_h1[j];
                const dbl4 g2 = a.j_h2[j];
                const double2 g3 = a.j_h3[j];
                s_a[wid][lane] = Real<F64>::make4((R)(p.x - cx), (R)(p.y - cy), (R)(p.z - cz), (R)p.w);
                const R hx = (R)(v.x - cvx), hy = (R)(v.y - cvy), hz = (R)(v.z - cvz);
                s_b[wid][lane] = Real<F64>::make4(hx, hy, hz, (R)g1.x);
                s_c[wid][lane] = Real<F64>::make4((R)(g1.y - cp), (R)g1.z, (R)g1.w, (R)g2.x);
                s_d[wid][lane] = Real<F64>::make4((R)g2.y, (R)g2.z, (R)g2.w, (R)(g3.x - cu));
                s_e[wid][lane] = Real<F64>::make4((R)g3.y, (R)(g1.x * g1.x * g1.x * g1.x),
                                                  (R)((v.x - cvx) - (double)hx), (R)((v.y - cvy) - (double)hy));
                s_f[wid][lane] = (R)((v.z - cvz) - (double)hz);
                s_id[wid][lane] = a.j_id[j];
            }
            __syncwarp();
            const int n = min(32, nj - t);
            R pax = 0, pay = 0, paz = 0, pud = 0, pdf = 0, pgx = 0, pgy = 0, pgz = 0;
            for (int k = sub; k < n; k += tpi) {
                const R4 A = s_a[wid][k];
                const R4 B = s_b[wid][k];
                const R4 C = s_c[wid][k];
                const R4 D = s_d[wid][k];
                const R4 E = s_e[wid][k];
                const R dx = xi - A.x, dy = yi - A.y, dz = zi - A.z;
                R ux = vxi - B.x, uy = vyi - B.y, uz = vzi - B.z;
                if (!F64) {
                    ux += lxi - E.z;
                    uy += lyi - E.w;
                    uz += lzi - s_f[wid][k];
                }
                const R r2 = dx * dx + dy * dy + dz * dz;
                const R ri = (idi != s_id[wid][k]) ? rsqrt_r(r2) : (R)0;
                const R r = r2 * ri;
                // kernel gradients W1(q) for both smoothing lengths
                const R qi = r * hi_i, qj = r * B.w;
                const R ui = max0((R)1 - qi), uj = max0((R)1 - qj);
                const R ui2 = ui * ui, uj2 = uj * uj;
                const R w1i = ui2 * (ui2 - ui * ((R)1 + (R)4 * qi));
                const R w1j = uj2 * (uj2 - uj * ((R)1 + (R)4 * qj));
                const R dw_i = (R)CEFF1 * hi4_i * w1i;
                const R dw_j = (R)CEFF1 * E.y * w1j;
                const R ka = (dw_i + dw_j) * A.w;
                // viscosity, hdr_hydro.hpp:368-376
                const R w = (dx * ux + dy * uy + dz * uz) * ri;
                const R wneg = w < (R)0 ? w : (R)0;
                const R vs = cs_i + D.x - (R)3 * wneg;
                const R rhi = rcp_r(dn_i + C.w);
                const R av = (bs_i + C.z) * (al_i + D.y) * vs * wneg;
                vsmx = vs > vsmx ? vs : vsmx;
                // pressure gradient, :378-382
                const R ta = (pc_i + C.y - (R)0.5 * av * rhi) * ka * ri;
                pax -= ta * dx;
                pay -= ta * dy;
                paz -= ta * dz;
                // energy equation with conduction, :384-393
                const R vsu2 = fabs(pp_i - C.x) * rhi * (R)2;
                const R vsu = vsu2 > (R)0 ? vsu2 * rsqrt_r(vsu2) : (R)0;
                const R du = eg_i - D.w;
                pud += ka * (pc_i * w - rhi * ((R)0.25 * av * wneg - (au_i + D.z) * vsu * du));
                pdf += rhi * du * ka * ri;
                // softening correction, :395-398
                const R dg = A.w * ri * (et_i * dw_i + E.x * dw_j);
                pgx += dg * dx;
                pgy += dg * dy;
                pgz += dg * dz;
            }
            ax.add(pax);
            ay.add(pay);
            az.add(paz);
            ud.add(pud);
            df.add(pdf);
            gx.add(pgx);
            gy.add(pgy);
            gz.add(pgz);
            __syncwarp();
        }
        const double sax = seg_sum(ax.value(), tpi), say = seg_sum(ay.value(), tpi);
        const double saz = seg_sum(az.value(), tpi), sud = seg_sum(ud.value(), tpi);
        const double sdf = seg_sum(df.value(), tpi), sgx = seg_sum(gx.value(), tpi);
        const double sgy = seg_sum(gy.value(), tpi), sgz = seg_sum(gz.value(), tpi);
        const double svs = seg_max((double)vsmx, tpi);
        if (act && sub == 0) {
            a.o_acch[3 * ii + 0] = 0.5 * sax;
            a.o_acch[3 * ii + 1] = 0.5 * say;
            a.o_acch[3 * ii + 2] = 0.5 * saz;
            a.o_accg[3 * ii + 0] = 0.5 * sgx;
            a.o_accg[3 * ii + 1] = 0.5 * sgy;
            a.o_accg[3 * ii + 2] = 0.5 * sgz;
            a.o_udot[ii] = 0.5 * sud;
            a.o_vsmx[ii] = svs;
            a.o_diffu[ii] = 2.0 * sdf;
        }
        (void)hinv4_d;
    }
}

// ---------------------------------------------------------------- gravity
struct GravityArgs {
    const dbl4 *i_pe;    // x, y, z, eps2
    // j sources: index k < n_split reads (j_pm, j_eps2)[k]; k >= n_split reads
    // (s_pm, s_eps2)[k - n_split] (superparticles / tree-node monopoles)
    const dbl4 *j_pm;    // x, y, z, mass
    const double *j_eps2;
    const dbl4 *s_pm;
    const double *s_eps2;
    int n_split;
    const WorkItem *items;
    int n_items;
    const int *n_items_dev;
    const int *j_off;
    const int *j_idx;
    int *queue;
    double *o_acc;          // 3 per particle (assigned)
    double *o_pot, *o_eta;
};

template <bool F64, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
gravity_kernel(const GravityArgs a) {
    typedef typename Real<F64>::T R;
    typedef typename Real<F64>::T4 R4;
    __shared__ R4 s_p[WARPS][32];   // dx, dy, dz, mass
    __shared__ R s_e[WARPS][32];    // eps2
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int n_items = a.n_items_dev ? *a.n_items_dev : a.n_items;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.queue, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= n_items) return;
        const WorkItem it = a.items[item];
        const int jb = a.j_off[it.x];
        const int nj = a.j_off[it.x + 1] - jb;
        const int tpi = lanes_per_i(it.z);
        const int sh = ilog2_pow2(tpi);
        const int li = lane >> sh;
        const int sub = lane & (tpi - 1);
        const bool act = li < it.z;
        const int ii = it.y + (act ? li : 0);

        double cx = 0, cy = 0, cz = 0;
        if (!F64) {
            const dbl4 c = a.i_pe[it.y];
            cx = c.x; cy = c.y; cz = c.z;
        }
        const dbl4 pi = a.i_pe[ii];
        const R xi = (R)(pi.x - cx), yi = (R)(pi.y - cy), zi = (R)(pi.z - cz);
        const R e2i = (R)pi.w;
        Acc<F64> ax, ay, az, pt, et;
        for (int t = 0; t < nj; t += 32) {
            const int jk = t + lane;
            if (jk < nj) {
                const int j = a.j_idx ? a.j_idx[jb + jk] : jb + jk;
                dbl4 p;
                double e2;
                if (j < a.n_split) {
                    p = a.j_pm[j];
                    e2 = a.j_eps2[j];
                } else {
                    p = a.s_pm[j - a.n_split];
                    e2 = a.s_eps2[j - a.n_split];
                }
                s_p[wid][lane] = Real<F64>::make4((R)(p.x - cx), (R)(p.y - cy), (R)(p.z - cz), (R)p.w);
                s_e[wid][lane] = (R)e2;
            }
            __syncwarp();
            const int n = min(32, nj - t);
            R pax = 0, pay = 0, paz = 0, ppt = 0, pet = 0;
            for (int k = sub; k < n; k += tpi) {
                const R4 pj = s_p[wid][k];
                const R dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
                const R r2 = dx * dx + dy * dy + dz * dz;
                const R rei = rsqrt_r(r2 + e2i);
                const R rej = rsqrt_r(r2 + s_e[wid][k]);
                const R rei3 = rei * rei * rei;
                const R rej3 = rej * rej * rej;
                const R g = pj.w * (rei3 + rej3);
                ppt -= pj.w * (rei + rej);
                pax -= dx * g;
                pay -= dy * g;
                paz -= dz * g;
                pet += pj.w * rei3;
            }
            ax.add(pax);
            ay.add(pay);
            az.add(paz);
            pt.add(ppt);
            et.add(pet);
            __syncwarp();
        }
        const double sax = seg_sum(ax.value(), tpi), say = seg_sum(ay.value(), tpi);
        const double saz = seg_sum(az.value(), tpi), spt = seg_sum(pt.value(), tpi);
        const double set = seg_sum(et.value(), tpi);
        if (act && sub == 0) {
            a.o_acc[3 * ii + 0] = 0.5 * sax;
            a.o_acc[3 * ii + 1] = 0.5 * say;
            a.o_acc[3 * ii + 2] = 0.5 * saz;
            a.o_pot[ii] = 0.5 * spt;
            a.o_eta[ii] = set;
        }
    }
}

}  // namespace sphk
