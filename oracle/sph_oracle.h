/*
 * sph_oracle.h — CPU oracle for the SPH interaction path (TEST INFRASTRUCTURE).
 *
 * Plain scalar FP64 C restatement of the reference's CPU functors
 * (yamauchi1132/Research_Codes, sph_yamauchi/run, USE_HELMHOLTZ build without
 * USE_INTRINSICS).  Only the tests, the smoke check and the CPU-baseline leg of
 * bench.py use it, always as the oracle or the timed CPU reference; the
 * product library never links it.
 *
 * Parity of this restatement is pinned against the reference's own functors
 * compiled from their source (oracle/Makefile target `ref`, see ref_bridge.cpp)
 * through the golden vectors under tests/golden/.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>
#include "../include/sph_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Wendland C2 3-D constants, hdr_kernel.hpp:218-227. */
#define ORACLE_KSRH  1.936492
#define ORACLE_CEFF0 3.342253804929802286e+00
#define ORACLE_CEFF1 1.336901521971920914e+01

/* calcDensity (hdr_density.hpp:246-366).  ksr_max <= 0 disables the clamp. */
void oracle_density(const sph_DensityEPI *epi, int32_t ni,
                    const sph_DensityEPJ *epj, int32_t nj,
                    sph_Density *out, double eta, double ksr_max);

/* calcHydro (hdr_hydro.hpp:312-424). */
void oracle_hydro(const sph_HydroEPI *epi, int32_t ni,
                  const sph_HydroEPJ *epj, int32_t nj, sph_Hydro *out);

/* calcGravity<TJ> (hdr_gravity.hpp:286-342), accumulating into out. */
void oracle_gravity_ep(const sph_GravityEPI *epi, int32_t ni,
                       const sph_GravityEPJ *epj, int32_t nj, sph_Gravity *out);
void oracle_gravity_sp(const sph_GravityEPI *epi, int32_t ni,
                       const sph_GravitySPJ *spj, int32_t nj, sph_Gravity *out);

/* Many walks at once, OpenMP over walks (the CPU baseline's threading).
 * Walk w owns epi[i_off[w] .. i_off[w+1]) and epj[j_off[w] .. j_off[w+1]).
 * Gravity assigns: out is cleared per walk before the sum (as Retrieve does).
 * nthreads <= 0 uses the OpenMP default.  Returns the thread count used. */
int oracle_density_walks(int32_t n_walk, const int64_t *i_off, const int64_t *j_off,
                         const sph_DensityEPI *epi, const sph_DensityEPJ *epj,
                         sph_Density *out, double eta, double ksr_max, int nthreads);
int oracle_hydro_walks(int32_t n_walk, const int64_t *i_off, const int64_t *j_off,
                       const sph_HydroEPI *epi, const sph_HydroEPJ *epj,
                       sph_Hydro *out, int nthreads);
int oracle_gravity_walks(int32_t n_walk, const int64_t *i_off, const int64_t *j_off,
                         const sph_GravityEPI *epi, const sph_GravityEPJ *epj,
                         sph_Gravity *out, int nthreads);

/* ---- per-particle step glue (FP64), arrays of length n ---------------- */

/* Ideal-gas EOS with n = 1.5 (hdr_hgas.hpp:318-344):
 * P = rho u / n, c = sqrt((1 + 1/n) P / rho). */
void oracle_eos(int64_t n, const double *dens, const double *uene,
                double *pres, double *vsnd);

/* Balsara switch (hdr_sph.hpp:79-89). */
void oracle_balsara(int64_t n, const double *divv, const double *rotv,
                    const double *vsnd, const double *ksr, double *bswt);

/* alpha / alpha_u time derivatives (hdr_hgas.hpp:750-762) with umin = 0 and
 * EpsilonOfInternalEnergy = eps_u. */
void oracle_alpha_dot(int64_t n, const double *divv, const double *alph,
                      const double *alphu, const double *vsnd, const double *ksr,
                      const double *uene, const double *diffu,
                      double alpha_max, double alpha_min,
                      double alphu_max, double alphu_min, double eps_u,
                      double *adot, double *adotu);

/* Per-particle time step (hdr_hgas.hpp:477-488); returns the minimum of
 * dt_max and all particles' limits. */
double oracle_timestep_min(int64_t n, const double *ksr, const double *vsmx,
                           const double *divv, const double *accg,  /* n*3 */
                           double c_dt, double dt_max);

/* sumAcceleration (hdr_sph.hpp:95-97), n x 3 arrays. */
void oracle_sum_acceleration(int64_t n, const double *acch, const double *accg1,
                             const double *accg2, double *acc);

/* Leapfrog predictor and corrector (hdr_hgas.hpp:646-665), in place. */
void oracle_predict(int64_t n, double dt, double *pos, double *vel, const double *acc,
                    double *vel2, double *uene, double *uene2, const double *udot,
                    double *alph, double *alph2, const double *adot,
                    double *alphu, double *alphu2, const double *adotu);
void oracle_correct(int64_t n, double dt, double *vel, const double *vel2, const double *acc,
                    double *uene, const double *uene2, const double *udot,
                    double *alph, const double *alph2, const double *adot,
                    double *alphu, const double *alphu2, const double *adotu);

/* Total energy (main.cpp:199-219, hdr_hgas.hpp:630-634); parts: optional
 * {kinetic, thermal, potential}. */
double oracle_energy(int64_t n, const double *mass, const double *vel, const double *uene,
                     const double *pot, double *parts);

/* Centre of mass of star `star` (< 0: all), hdr_util.hpp:8-34;
 * out = {m, x, y, z, vx, vy, vz}. */
void oracle_center_of_mass(int64_t n, const double *mass, const double *pos, const double *vel,
                           const int32_t *istar, int32_t star, double *out);

/* Maximum kernel support radius (hdr_util.hpp:489-506, FlagBinary 0). */
double oracle_ksrmax(int64_t n, const double *mass, const double *pos, const double *vel,
                     const int32_t *istar, const double *dens);

/* Power-of-two global time step (main.cpp:242-273); < 0 where the
 * reference aborts (dt would fall to dt_min). */
double oracle_timestep_pow2(double dt, double dtc, double time, double dt_max, double dt_min);

/* Host octree over Morton-sorted particles and theta-criterion gravity lists
 * per i-group (the CPU arm's stand-in for FDPS's TreeForForceLong walk).
 * Call with null ep_idx/sp_idx/node arrays to get the offsets and the node
 * count, then again to fill. */
int64_t oracle_gravity_lists(int64_t n, const uint64_t *keys, const double *pos, const double *mass,
                             const double *eps2, int32_t ng, const int64_t *gfirst, const int64_t *gcount,
                             double theta, int32_t n_leaf, int64_t *ep_off, int64_t *sp_off,
                             int32_t *ep_idx, int32_t *sp_idx, double *node_mom, double *node_eps2,
                             int nthreads);
void oracle_neighbour_lists(int64_t n, const uint64_t *keys, const double *pos, const double *h, int32_t ng,
                            const int64_t *gfirst, const int64_t *gcount, const double *gr, int32_t mode,
                            int32_t n_leaf, int64_t *off, int32_t *idx, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
