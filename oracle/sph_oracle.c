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
