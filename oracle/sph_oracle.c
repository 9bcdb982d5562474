/*
 * sph_oracle.c — CPU oracle for the SPH interaction path (TEST INFRASTRUCTURE).
 *
 * Scalar FP64 restatement of the reference's CPU functors of
 * yamauchi1132/Research_Codes (sph_yamauchi/run, USE_HELMHOLTZ, no
 * USE_INTRINSICS).  Each function names the reference lines it follows.  Only
 * tests, the smoke check and bench.py's CPU-baseline leg call this code.
 */
#include "sph_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Wendland C2 in 3-D and its radial derivative term, hdr_kernel.hpp:246-257:
 *   W0(q) = c0 (1-q)_+^4 (1+4q)
 *   W1(q) = c1 [(1-q)_+^4 - (1-q)_+^3 (1+4q)]                              */
static inline double wendland_w0(double q) {
    double t = 1.0 - q;
    if (!(t > 0.0)) t = 0.0;
    double t2 = t * t;
    return ORACLE_CEFF0 * t2 * t2 * (1.0 + 4.0 * q);
}

static inline double wendland_w1(double q) {
    double t = 1.0 - q;
    if (!(t > 0.0)) t = 0.0;
    double t2 = t * t;
    return ORACLE_CEFF1 * (t2 * t2 - t2 * t * (1.0 + 4.0 * q));
}

/* calcDensity::operator(), hdr_density.hpp:254-363.
 * Three fixed-point passes over the same j-list: rho from the current h,
 * then h <- min(eta ksrh (m/rho)^(1/3), ksrmax) (:264-302).  The stored rho and
 * np are those of the third pass (computed with the second pass's h) and the
 * stored h is the third update.  A fourth pass with the final h gives
 * grad-h, div v and rot v (:304-349), normalised by rho and Omega (:351-362). */
void oracle_density(const sph_DensityEPI *epi, int32_t ni,
                    const sph_DensityEPJ *epj, int32_t nj,
                    sph_Density *out, double eta, double ksr_max) {
    const double hmax = (ksr_max > 0.0) ? ksr_max : INFINITY;
    for (int32_t i = 0; i < ni; ++i) {
        const sph_DensityEPI *pi = &epi[i];
        double h = pi->ksr;
        for (int pass = 0; pass < 3; ++pass) {
            const double hinv = 1.0 / h;
            const double hinv3 = hinv * hinv * hinv;
            double rho = 0.0;
            int64_t cnt = 0;
            for (int32_t j = 0; j < nj; ++j) {
                const double dx = pi->pos[0] - epj[j].pos[0];
                const double dy = pi->pos[1] - epj[j].pos[1];
                const double dz = pi->pos[2] - epj[j].pos[2];
                const double q = sqrt(dx * dx + dy * dy + dz * dz) * hinv;
                rho += epj[j].mass * hinv3 * wendland_w0(q);
                cnt += (q < 1.0) ? 1 : 0;
            }
            double hn = eta * ORACLE_KSRH * pow(pi->mass / rho, 1.0 / 3.0);
            hn = (hn < hmax) ? hn : hmax;
            out[i].dens = rho;
            out[i].np = cnt;
            out[i].ksr = hn;
            out[i].itr = (hn > pi->rs);
            h = hn;
        }

        const double hinv = 1.0 / h;
        const double hinv4 = hinv * hinv * hinv * hinv;
        double grdh = 0.0, divv = 0.0, rx = 0.0, ry = 0.0, rz = 0.0;
        for (int32_t j = 0; j < nj; ++j) {
            const double dx = pi->pos[0] - epj[j].pos[0];
            const double dy = pi->pos[1] - epj[j].pos[1];
            const double dz = pi->pos[2] - epj[j].pos[2];
            const double ux = pi->vel[0] - epj[j].vel[0];
            const double uy = pi->vel[1] - epj[j].vel[1];
            const double uz = pi->vel[2] - epj[j].vel[2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            /* self pair (same id) gets 1/r = 0, hdr_density.hpp:320-321 */
            const double rinv = ((int64_t)pi->id != (int64_t)epj[j].id) ? 1.0 / sqrt(r2) : 0.0;
            const double q = r2 * rinv * hinv;
            const double w0 = wendland_w0(q);
            const double w1 = wendland_w1(q);
            const double m = epj[j].mass;
            grdh -= (3.0 * w0 + q * w1) * hinv4 * m;
            const double dw = m * hinv4 * w1 * rinv;
            const double gx = dw * dx, gy = dw * dy, gz = dw * dz;
            divv -= ux * gx + uy * gy + uz * gz;
            rx += uy * gz - uz * gy;
            ry += uz * gx - ux * gz;
            rz += ux * gy - uy * gx;
        }
        const double rho = out[i].dens;
        const double rhoinv = 1.0 / rho;
        const double omega = 1.0 / (1.0 + h * rhoinv * grdh / 3.0);
        const double rot2 = rx * rx + ry * ry + rz * rz;
        const double rot = (rot2 != 0.0) ? rot2 / sqrt(rot2) : 0.0;
        out[i].divv = divv * rhoinv * omega;
        out[i].rotv = rot * rhoinv * omega;
        out[i].grdh = omega;
    }
}

/* calcHydro::operator(), hdr_hydro.hpp:320-421. */
void oracle_hydro(const sph_HydroEPI *epi, int32_t ni,
                  const sph_HydroEPJ *epj, int32_t nj, sph_Hydro *out) {
    for (int32_t i = 0; i < ni; ++i) {
        const sph_HydroEPI *a = &epi[i];
        const double hinv4_i = a->hinv * a->hinv * a->hinv * a->hinv;
        double ax = 0.0, ay = 0.0, az = 0.0, udot = 0.0, vsmx = 0.0, difu = 0.0;
        double gx = 0.0, gy = 0.0, gz = 0.0;
        for (int32_t j = 0; j < nj; ++j) {
            const sph_HydroEPJ *b = &epj[j];
            const double dx = a->pos[0] - b->pos[0];
            const double dy = a->pos[1] - b->pos[1];
            const double dz = a->pos[2] - b->pos[2];
            const double ux = a->vel[0] - b->vel[0];
            const double uy = a->vel[1] - b->vel[1];
            const double uz = a->vel[2] - b->vel[2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double rinv = (a->id != b->id) ? 1.0 / sqrt(r2) : 0.0;
            const double r = r2 * rinv;
            const double hinv4_j = b->hinv * b->hinv * b->hinv * b->hinv;
            const double dw_i = hinv4_i * wendland_w1(r * a->hinv);
            const double dw_j = hinv4_j * wendland_w1(r * b->hinv);
            const double ka = (dw_i + dw_j) * b->mass;

            /* artificial viscosity with the Balsara switch (:368-374) */
            const double w = (dx * ux + dy * uy + dz * uz) * rinv;
            const double wneg = (w < 0.0) ? w : 0.0;
            const double vsig = a->vsnd + b->vsnd - 3.0 * wneg;
            const double rhobar_inv = 1.0 / (a->dens + b->dens);
            const double av = (a->bswt + b->bswt) * (a->alph + b->alph) * vsig * wneg;
            vsmx = (vsmx > vsig) ? vsmx : vsig;

            /* pressure gradient + viscosity (:378-382) */
            const double fa = (a->presc + b->presc - 0.5 * av * rhobar_inv) * ka * rinv;
            ax -= fa * dx;
            ay -= fa * dy;
            az -= fa * dz;

            /* du/dt with the thermal-conduction signal velocity (:384-391) */
            const double vsu2 = fabs(a->pres - b->pres) * rhobar_inv * 2.0;
            const double vsu = (vsu2 != 0.0) ? vsu2 / sqrt(vsu2) : 0.0;
            const double du = a->thrm - b->thrm;
            udot += ka * (a->presc * w
                          - rhobar_inv * (0.25 * av * wneg - (a->alphu + b->alphu) * vsu * du));
            difu += rhobar_inv * du * ka * rinv;

            /* gravity-softening correction (:395-398) */
            const double dg = b->mass * rinv * (a->eta * dw_i + b->eta * dw_j);
            gx += dg * dx;
            gy += dg * dy;
            gz += dg * dz;
        }
        out[i].acch[0] = 0.5 * ax;
        out[i].acch[1] = 0.5 * ay;
        out[i].acch[2] = 0.5 * az;
        out[i].udot = 0.5 * udot;
        out[i].vsmx = vsmx;
        out[i].diffu = 2.0 * difu;
        out[i].accg[0] = 0.5 * gx;
        out[i].accg[1] = 0.5 * gy;
        out[i].accg[2] = 0.5 * gz;
    }
}

/* calcGravity<TJ>::operator(), hdr_gravity.hpp:295-339: symmetrised Plummer
 * softening, R_k = (r^2 + eps_k^2)^(-1/2); pot -= m/2 (R_i + R_j),
 * a -= m/2 (R_i^3 + R_j^3) dx, eta += m R_i^3.  Accumulates. */
static void gravity_core(const sph_GravityEPI *epi, int32_t ni,
                         const double *j_mass_pos_eps2, int32_t nj, size_t stride,
                         sph_Gravity *out) {
    for (int32_t i = 0; i < ni; ++i) {
        const sph_GravityEPI *a = &epi[i];
        double ax = 0.0, ay = 0.0, az = 0.0, pot = 0.0, eta = 0.0;
        for (int32_t j = 0; j < nj; ++j) {
            const double *b = j_mass_pos_eps2 + (size_t)j * stride;
            const double m = b[0];
            const double dx = a->pos[0] - b[1];
            const double dy = a->pos[1] - b[2];
            const double dz = a->pos[2] - b[3];
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double ri = 1.0 / sqrt(r2 + a->eps2);
            const double rj = 1.0 / sqrt(r2 + b[4]);
            const double ri3 = ri * ri * ri;
            const double rj3 = rj * rj * rj;
            const double g = m * (ri3 + rj3);
            pot -= m * (ri + rj);
            ax -= dx * g;
            ay -= dy * g;
            az -= dz * g;
            eta += m * ri3;
        }
        out[i].acc[0] += 0.5 * ax;
        out[i].acc[1] += 0.5 * ay;
        out[i].acc[2] += 0.5 * az;
        out[i].pot += 0.5 * pot;
        out[i].eta += eta;
    }
}

void oracle_gravity_ep(const sph_GravityEPI *epi, int32_t ni,
                       const sph_GravityEPJ *epj, int32_t nj, sph_Gravity *out) {
    gravity_core(epi, ni, (const double *)epj, nj, sizeof(sph_GravityEPJ) / sizeof(double), out);
}

void oracle_gravity_sp(const sph_GravityEPI *epi, int32_t ni,
                       const sph_GravitySPJ *spj, int32_t nj, sph_Gravity *out) {
    gravity_core(epi, ni, (const double *)spj, nj, sizeof(sph_GravitySPJ) / sizeof(double), out);
}

static int set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

int oracle_density_walks(int32_t n_walk, const int64_t *i_off, const int64_t *j_off,
                         const sph_DensityEPI *epi, const sph_DensityEPJ *epj,
                         sph_Density *out, double eta, double ksr_max, int nthreads) {
    int nt = set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t w = 0; w < n_walk; ++w) {
        oracle_density(epi + i_off[w], (int32_t)(i_off[w + 1] - i_off[w]),
                       epj + j_off[w], (int32_t)(j_off[w + 1] - j_off[w]),
                       out + i_off[w], eta, ksr_max);
    }
    return nt;
}

int oracle_hydro_walks(int32_t n_walk, const int64_t *i_off, const int64_t *j_off,
                       const sph_HydroEPI *epi, const sph_HydroEPJ *epj,
                       sph_Hydro *out, int nthreads) {
    int nt = set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t w = 0; w < n_walk; ++w) {
        oracle_hydro(epi + i_off[w], (int32_t)(i_off[w + 1] - i_off[w]),
                     epj + j_off[w], (int32_t)(j_off[w + 1] - j_off[w]),
                     out + i_off[w]);
    }
    return nt;
}

int oracle_gravity_walks(int32_t n_walk, const int64_t *i_off, const int64_t *j_off,
                         const sph_GravityEPI *epi, const sph_GravityEPJ *epj,
                         sph_Gravity *out, int nthreads) {
    int nt = set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t w = 0; w < n_walk; ++w) {
        const int32_t ni = (int32_t)(i_off[w + 1] - i_off[w]);
        memset(out + i_off[w], 0, sizeof(sph_Gravity) * (size_t)ni);
        oracle_gravity_ep(epi + i_off[w], ni, epj + j_off[w],
                          (int32_t)(j_off[w + 1] - j_off[w]), out + i_off[w]);
    }
    return nt;
}

/* ---- step glue ---------------------------------------------------------- */

void oracle_eos(int64_t n, const double *dens, const double *uene,
                double *pres, double *vsnd) {
    const double ninv = 1.0 / 1.5;                      /* hdr_hgas.hpp:767-768 */
    for (int64_t i = 0; i < n; ++i) {
        pres[i] = ninv * dens[i] * uene[i];             /* hdr_hgas.hpp:339 */
        vsnd[i] = sqrt((1.0 + ninv) * pres[i] / dens[i]); /* hdr_hgas.hpp:341 */
    }
}

void oracle_balsara(int64_t n, const double *divv, const double *rotv,
                    const double *vsnd, const double *ksr, double *bswt) {
    for (int64_t i = 0; i < n; ++i) {                   /* hdr_sph.hpp:79-81 */
        const double ad = fabs(divv[i]);
        bswt[i] = ad / (ad + fabs(rotv[i]) + 1e-4 * vsnd[i] * ORACLE_KSRH / ksr[i]);
    }
}

void oracle_alpha_dot(int64_t n, const double *divv, const double *alph,
                      const double *alphu, const double *vsnd, const double *ksr,
                      const double *uene, const double *diffu,
                      double alpha_max, double alpha_min,
                      double alphu_max, double alphu_min, double eps_u,
                      double *adot, double *adotu) {
    for (int64_t i = 0; i < n; ++i) {                   /* hdr_hgas.hpp:750-762 */
        double src = -divv[i] * (alpha_max - alph[i]);
        if (src < 0.0) src = 0.0;
        const double tauinv = (0.25 * ORACLE_KSRH * vsnd[i]) / ksr[i];
        adot[i] = -(alph[i] - alpha_min) * tauinv + src;
        double u = uene[i];                             /* umin = 0 */
        if (u < 0.0) u = 0.0;
        double room = alphu_max - alphu[i];
        if (room < 0.0) room = 0.0;
        const double srcu = ksr[i] / ORACLE_KSRH * fabs(diffu[i]) / sqrt(u + eps_u) * room;
        adotu[i] = -(alphu[i] - alphu_min) * tauinv + srcu;
    }
}

double oracle_timestep_min(int64_t n, const double *ksr, const double *vsmx,
                           const double *divv, const double *accg,
                           double c_dt, double dt_max) {
    double dtc = dt_max;                                /* main.cpp:244-249 */
    for (int64_t i = 0; i < n; ++i) {                   /* hdr_hgas.hpp:477-488 */
        const double dth = c_dt * ksr[i] / (vsmx[i] * ORACLE_KSRH);
        const double dtd = (divv[i] < 0.0) ? (-c_dt / divv[i]) : dt_max;
        const double g = sqrt(accg[3 * i] * accg[3 * i] + accg[3 * i + 1] * accg[3 * i + 1]
                              + accg[3 * i + 2] * accg[3 * i + 2]);
        const double dtg = c_dt * sqrt(ksr[i] / g);
        double d = dt_max;
        if (dth < d) d = dth;
        if (dtg < d) d = dtg;
        if (dtd < d) d = dtd;
        if (d < dtc) dtc = d;
    }
    return dtc;
}

/* sumAcceleration (hdr_sph.hpp:95-97): a = a_h + a_g1 + a_g2 (n x 3). */
void oracle_sum_acceleration(int64_t n, const double *acch, const double *accg1,
                             const double *accg2, double *acc) {
    for (int64_t k = 0; k < 3 * n; ++k) acc[k] = acch[k] + accg1[k] + accg2[k];
}

/* HelmholtzGas::predict (hdr_hgas.hpp:646-657) with dnuc = 0 (no nuclear
 * network) and without the Paczynski-Wiita gcor3 channel: in place. */
void oracle_predict(int64_t n, double dt, double *pos, double *vel, const double *acc,
                    double *vel2, double *uene, double *uene2, const double *udot,
                    double *alph, double *alph2, const double *adot,
                    double *alphu, double *alphu2, const double *adotu) {
    for (int64_t i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) {
            const int64_t k = 3 * i + c;
            pos[k] = pos[k] + vel[k] * dt + 0.5 * acc[k] * dt * dt;
            vel2[k] = vel[k] + 0.5 * acc[k] * dt;
            vel[k] = vel[k] + acc[k] * dt;
        }
        uene2[i] = uene[i] + 0.5 * udot[i] * dt;
        uene[i] = uene[i] + udot[i] * dt;
        alph2[i] = alph[i] + 0.5 * adot[i] * dt;
        alph[i] = alph[i] + adot[i] * dt;
        alphu2[i] = alphu[i] + 0.5 * adotu[i] * dt;
        alphu[i] = alphu[i] + adotu[i] * dt;
    }
}

/* HelmholtzGas::correct (hdr_hgas.hpp:659-665), dnuc = 0: in place. */
void oracle_correct(int64_t n, double dt, double *vel, const double *vel2, const double *acc,
                    double *uene, const double *uene2, const double *udot,
                    double *alph, const double *alph2, const double *adot,
                    double *alphu, const double *alphu2, const double *adotu) {
    for (int64_t i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) vel[3 * i + c] = vel2[3 * i + c] + 0.5 * acc[3 * i + c] * dt;
        uene[i] = uene2[i] + 0.5 * udot[i] * dt;
        alph[i] = alph2[i] + 0.5 * adot[i] * dt;
        alphu[i] = alphu2[i] + 0.5 * adotu[i] * dt;
    }
}

/* calcEnergy (main.cpp:199-219) over HelmholtzGas::calcEnergy
 * (hdr_hgas.hpp:630-634), gcor3 = 0: sum m (v^2/2 + u + pot/2), summed in
 * index order.  parts[3] (optional) receives the kinetic, thermal and
 * potential sums. */
double oracle_energy(int64_t n, const double *mass, const double *vel, const double *uene,
                     const double *pot, double *parts) {
    double e = 0.0, ek = 0.0, eu = 0.0, ep = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double *v = vel + 3 * i;
        const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        e += mass[i] * (0.5 * v2 + uene[i] + 0.5 * pot[i]);
        ek += mass[i] * 0.5 * v2;
        eu += mass[i] * uene[i];
        ep += mass[i] * 0.5 * pot[i];
    }
    if (parts) {
        parts[0] = ek;
        parts[1] = eu;
        parts[2] = ep;
    }
    return e;
}

/* calcCenterOfMass (hdr_util.hpp:8-34): mass, centre of mass and its velocity
 * over the particles of star `star` (all particles when star < 0).
 * out = {m, x, y, z, vx, vy, vz}. */
void oracle_center_of_mass(int64_t n, const double *mass, const double *pos, const double *vel,
                           const int32_t *istar, int32_t star, double *out) {
    double m = 0.0, x[3] = {0.0, 0.0, 0.0}, v[3] = {0.0, 0.0, 0.0};
    for (int64_t i = 0; i < n; ++i) {
        if (star >= 0 && istar[i] != star) continue;
        m += mass[i];
        for (int c = 0; c < 3; ++c) {
            x[c] += mass[i] * pos[3 * i + c];
            v[c] += mass[i] * vel[3 * i + c];
        }
    }
    const double minv = 1.0 / m;
    out[0] = m;
    for (int c = 0; c < 3; ++c) {
        out[1 + c] = x[c] * minv;
        out[4 + c] = v[c] * minv;
    }
}

/* calcKernelSupportRadiusMaximum (hdr_util.hpp:489-506, FlagBinary 0): the
 * density-weighted rms distance from star 0's centre of mass,
 * sqrt(sum rho |x - x_c|^2 / sum rho) over all particles. */
double oracle_ksrmax(int64_t n, const double *mass, const double *pos, const double *vel,
                     const int32_t *istar, const double *dens) {
    double c[7];
    oracle_center_of_mass(n, mass, pos, vel, istar, 0, c);
    double r2 = 0.0, dn = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double dx = pos[3 * i] - c[1], dy = pos[3 * i + 1] - c[2], dz = pos[3 * i + 2] - c[3];
        r2 += dens[i] * (dx * dx + dy * dy + dz * dz);
        dn += dens[i];
    }
    return sqrt(r2 / dn);
}

/* The global time step of calcTimestep (main.cpp:242-273): from the previous
 * step dt (RP::Timestep) and the particles' minimum dtc, halve while
 * dt > dtc (failing at dt <= dt_min, where the reference aborts), or double
 * when 2 dt <= dtc, 2 dt <= dt_max and the time is a multiple of 2 dt.
 * Returns the new dt, or a negative value where the reference aborts. */
double oracle_timestep_pow2(double dt, double dtc, double time, double dt_max, double dt_min) {
    if (dt > dtc) {
        while (dt > dtc) {
            dt *= 0.5;
            if (dt <= dt_min) return -1.0;
        }
    } else if (2.0 * dt <= dtc && 2.0 * dt <= dt_max) {
        const double dt2 = 2.0 * dt;
        if (time - (double)(int64_t)(time / dt2) * dt2 == 0.0) dt *= 2.0;
    }
    return dt;
}

/* ---- host tree and theta-criterion gravity lists ------------------------
 * The reference gets its gravity lists from FDPS's TreeForForceLong walk
 * (hdr_gravity.hpp:385-402, theta from the run parameters, n_group i-groups,
 * main.cpp:380-394); FDPS is not part of the reference tree.  This is a
 * plain octree of the same kind for the CPU arm of the benchmark: particles
 * sorted by 63-bit Morton key, a node is a run of keys with a common prefix
 * of 3 bits per level, leaves hold <= n_leaf particles.  Node monopoles are
 * hdr_gravity.hpp:37-49's (mass, centre of mass, mass-weighted eps^2); a
 * node is accepted for a group when the squared distance from the group's
 * bounding box to the node's centre of mass exceeds (node size / theta)^2
 * (size: the largest side of the node's particle bounding box), otherwise
 * opened; leaves that are not accepted enter as particles. */
typedef struct {
    int64_t first, count;
    int32_t child0, nchild;   /* children: consecutive node indices */
    double com[3], mass, eps2, size;
    double lo[3], hi[3], hmax; /* particle bounding box, largest h (neighbour lists) */
} otree_node;

typedef struct {
    otree_node *nodes;
    int64_t n_nodes, cap;
    int32_t *kids;            /* scratch for child lists */
} otree;

static int64_t key_bound(const uint64_t *keys, int64_t lo, int64_t hi, uint64_t v) {
    while (lo < hi) {         /* first index in [lo, hi) with keys >= v */
        const int64_t mid = lo + (hi - lo) / 2;
        if (keys[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

static int64_t otree_push(otree *t) {
    if (t->n_nodes == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 1024;
        t->nodes = (otree_node *)realloc(t->nodes, sizeof(otree_node) * (size_t)t->cap);
    }
    return t->n_nodes++;
}

/* node index v covers keys [first, first + count) sharing the key prefix above
 * bit 3 * (21 - level) */
static void otree_build(otree *t, int64_t v, const uint64_t *keys, const double *pos, const double *mass,
                        const double *eps2, int level, int n_leaf) {
    otree_node nd = t->nodes[v];
    double m = 0.0, c[3] = {0.0, 0.0, 0.0}, e = 0.0, lo[3], hi[3];
    for (int k = 0; k < 3; ++k) { lo[k] = 1e300; hi[k] = -1e300; }
    nd.hmax = 0.0;
    for (int64_t i = nd.first; i < nd.first + nd.count; ++i) {
        m += mass[i];
        e += mass[i] * eps2[i];
        for (int k = 0; k < 3; ++k) {
            const double x = pos[3 * i + k];
            c[k] += mass[i] * x;
            if (x < lo[k]) lo[k] = x;
            if (x > hi[k]) hi[k] = x;
        }
    }
    nd.mass = m;
    nd.eps2 = e / m;
    nd.size = 0.0;
    for (int k = 0; k < 3; ++k) {
        nd.com[k] = c[k] / m;
        nd.lo[k] = lo[k];
        nd.hi[k] = hi[k];
        if (hi[k] - lo[k] > nd.size) nd.size = hi[k] - lo[k];
    }
    nd.child0 = -1;
    nd.nchild = 0;
    t->nodes[v] = nd;
    if (nd.count <= n_leaf || level >= 21) return;
    const int shift = 3 * (20 - level);
    const uint64_t base = keys[nd.first] >> (shift + 3) << (shift + 3);
    int64_t starts[9];
    starts[0] = nd.first;
    for (int o = 1; o < 8; ++o) starts[o] = key_bound(keys, nd.first, nd.first + nd.count, base | ((uint64_t)o << shift));
    starts[8] = nd.first + nd.count;
    int32_t first_child = -1, nk = 0;
    for (int o = 0; o < 8; ++o) {
        if (starts[o + 1] == starts[o]) continue;
        const int64_t u = otree_push(t);
        t->nodes[u].first = starts[o];
        t->nodes[u].count = starts[o + 1] - starts[o];
        if (first_child < 0) first_child = (int32_t)u;
        ++nk;
    }
    t->nodes[v].child0 = first_child;
    t->nodes[v].nchild = nk;
    for (int32_t u = first_child; u < first_child + nk; ++u)
        otree_build(t, u, keys, pos, mass, eps2, level + 1, n_leaf);
}

/* Walk of group g: appends particle indices to ep (if non-null) and node
 * indices to sp; returns the counts. */
static void otree_walk(const otree *t, const double *glo, const double *ghi, double inv_theta2,
                       int32_t *ep, int64_t *nep, int32_t *sp, int64_t *nsp, int32_t *stack) {
    int64_t top = 0, ne = 0, ns = 0;
    stack[top++] = 0;
    while (top > 0) {
        const otree_node *nd = &t->nodes[stack[--top]];
        const int32_t v = (int32_t)(nd - t->nodes);
        double d2 = 0.0;
        for (int k = 0; k < 3; ++k) {
            double d = 0.0;
            if (nd->com[k] < glo[k]) d = glo[k] - nd->com[k];
            else if (nd->com[k] > ghi[k]) d = nd->com[k] - ghi[k];
            d2 += d * d;
        }
        if (d2 > nd->size * nd->size * inv_theta2) {
            if (sp) sp[ns] = v;
            ++ns;
        } else if (nd->nchild == 0) {
            for (int64_t i = nd->first; i < nd->first + nd->count; ++i) {
                if (ep) ep[ne] = (int32_t)i;
                ++ne;
            }
        } else {
            for (int32_t u = nd->child0 + nd->nchild - 1; u >= nd->child0; --u) stack[top++] = u;
        }
    }
    *nep = ne;
    *nsp = ns;
}

/* keys: sorted 63-bit Morton keys of pos (n x 3, same order); groups
 * [gfirst[g], gfirst[g] + gcount[g]).  Fills ep_off / sp_off (ng + 1) and,
 * when ep_idx / sp_idx are non-null, the lists; node_mom (4 per node: x, y,
 * z, mass) and node_eps2 when non-null.  Returns the node count (call once
 * with null outputs to size them). */
int64_t oracle_gravity_lists(int64_t n, const uint64_t *keys, const double *pos, const double *mass,
                             const double *eps2, int32_t ng, const int64_t *gfirst, const int64_t *gcount,
                             double theta, int32_t n_leaf, int64_t *ep_off, int64_t *sp_off,
                             int32_t *ep_idx, int32_t *sp_idx, double *node_mom, double *node_eps2,
                             int nthreads) {
    set_threads(nthreads);
    otree t = {0, 0, 0, 0};
    const int64_t root = otree_push(&t);
    t.nodes[root].first = 0;
    t.nodes[root].count = n;
    otree_build(&t, root, keys, pos, mass, eps2, 0, n_leaf);
    const double inv_theta2 = 1.0 / (theta * theta);
    const int fill = ep_idx != NULL;
#pragma omp parallel
    {
        int32_t *stack = (int32_t *)malloc(sizeof(int32_t) * (size_t)(8 * 22 + 64));
#pragma omp for schedule(dynamic, 4)
        for (int32_t g = 0; g < ng; ++g) {
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            for (int64_t i = gfirst[g]; i < gfirst[g] + gcount[g]; ++i)
                for (int k = 0; k < 3; ++k) {
                    if (pos[3 * i + k] < lo[k]) lo[k] = pos[3 * i + k];
                    if (pos[3 * i + k] > hi[k]) hi[k] = pos[3 * i + k];
                }
            int64_t ne, ns;
            if (fill)
                otree_walk(&t, lo, hi, inv_theta2, ep_idx + ep_off[g], &ne, sp_idx + sp_off[g], &ns, stack);
            else {
                otree_walk(&t, lo, hi, inv_theta2, NULL, &ne, NULL, &ns, stack);
                ep_off[g + 1] = ne;
                sp_off[g + 1] = ns;
            }
        }
        free(stack);
    }
    if (!fill) {
        ep_off[0] = sp_off[0] = 0;
        for (int32_t g = 0; g < ng; ++g) {
            ep_off[g + 1] += ep_off[g];
            sp_off[g + 1] += sp_off[g];
        }
    }
    if (node_mom)
        for (int64_t v = 0; v < t.n_nodes; ++v) {
            for (int k = 0; k < 3; ++k) node_mom[4 * v + k] = t.nodes[v].com[k];
            node_mom[4 * v + 3] = t.nodes[v].mass;
            if (node_eps2) node_eps2[v] = t.nodes[v].eps2;
        }
    const int64_t nn = t.n_nodes;
    free(t.nodes);
    return nn;
}

/* Largest h of every node (children before parents: children have larger
 * indices than their parent). */
static void otree_hmax(otree *t, const double *h) {
    for (int64_t v = t->n_nodes - 1; v >= 0; --v) {
        otree_node *nd = &t->nodes[v];
        double m = 0.0;
        if (nd->nchild == 0) {
            for (int64_t i = nd->first; i < nd->first + nd->count; ++i)
                if (h[i] > m) m = h[i];
        } else {
            for (int32_t u = nd->child0; u < nd->child0 + nd->nchild; ++u)
                if (t->nodes[u].hmax > m) m = t->nodes[u].hmax;
        }
        nd->hmax = m;
    }
}

static double box_d2(const double *alo, const double *ahi, const double *blo, const double *bhi) {
    double d2 = 0.0;
    for (int k = 0; k < 3; ++k) {
        double d = 0.0;
        if (blo[k] > ahi[k]) d = blo[k] - ahi[k];
        else if (alo[k] > bhi[k]) d = alo[k] - bhi[k];
        d2 += d * d;
    }
    return d2;
}

/* Gather and symmetric neighbour lists of groups (the roles of FDPS's
 * Gather search for the density, hdr_density.hpp:389-397, and its Symmetry
 * search for the hydro force, main.cpp:336-344), on the host octree above.
 * Group g covers particles [gfirst[g], gfirst[g] + gcount[g]) with bounding
 * box B_g and radius gr[g] (gr < 0: the group gets an empty list).
 *   mode 0: every particle j with dist(x_j, B_g) <= gr[g];
 *   mode 1: every particle j with dist(x_j, B_g) <= max(gr[g], h[j]).
 * Entries come in ascending particle order.  Fills off (ng + 1) and, when idx
 * is non-null, the lists (call once with idx null to size them). */
void oracle_neighbour_lists(int64_t n, const uint64_t *keys, const double *pos, const double *h, int32_t ng,
                            const int64_t *gfirst, const int64_t *gcount, const double *gr, int32_t mode,
                            int32_t n_leaf, int64_t *off, int32_t *idx, int nthreads) {
    set_threads(nthreads);
    double *unit = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) unit[i] = 1.0;
    otree t = {0, 0, 0, 0};
    const int64_t root = otree_push(&t);
    t.nodes[root].first = 0;
    t.nodes[root].count = n;
    otree_build(&t, root, keys, pos, unit, unit, 0, n_leaf);
    otree_hmax(&t, h);
    free(unit);
    const int fill = idx != NULL;
#pragma omp parallel
    {
        int32_t *stack = (int32_t *)malloc(sizeof(int32_t) * (size_t)(8 * 22 + 64));
#pragma omp for schedule(dynamic, 4)
        for (int32_t g = 0; g < ng; ++g) {
            int64_t ne = 0;
            if (gr[g] >= 0.0 && gcount[g] > 0) {
                double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
                for (int64_t i = gfirst[g]; i < gfirst[g] + gcount[g]; ++i)
                    for (int k = 0; k < 3; ++k) {
                        if (pos[3 * i + k] < lo[k]) lo[k] = pos[3 * i + k];
                        if (pos[3 * i + k] > hi[k]) hi[k] = pos[3 * i + k];
                    }
                int32_t *out = fill ? idx + off[g] : NULL;
                int64_t top = 0;
                stack[top++] = 0;
                while (top > 0) {
                    const otree_node *nd = &t.nodes[stack[--top]];
                    const double r = (mode == 1 && nd->hmax > gr[g]) ? nd->hmax : gr[g];
                    if (box_d2(lo, hi, nd->lo, nd->hi) > r * r) continue;
                    if (nd->nchild == 0) {
                        for (int64_t i = nd->first; i < nd->first + nd->count; ++i) {
                            const double ri = (mode == 1 && h[i] > gr[g]) ? h[i] : gr[g];
                            if (box_d2(lo, hi, pos + 3 * i, pos + 3 * i) > ri * ri) continue;
                            if (out) out[ne] = (int32_t)i;
                            ++ne;
                        }
                    } else {
                        for (int32_t u = nd->child0 + nd->nchild - 1; u >= nd->child0; --u) stack[top++] = u;
                    }
                }
            }
            if (!fill) off[g + 1] = ne;
        }
        free(stack);
    }
    if (!fill) {
        off[0] = 0;
        for (int32_t g = 0; g < ng; ++g) off[g + 1] += off[g];
    }
    free(t.nodes);
}
