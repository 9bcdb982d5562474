// ref_glue.cpp — the reference's own per-particle step glue behind a C ABI.
// TEST INFRASTRUCTURE: compiled by `make -C oracle ref` from the reference
// source tree (REF_DIR, read in place, never copied) into
// oracle/_ref/libsph_ref_glue.so.  The C restatement of the glue in
// sph_oracle.c is checked against it (tests/test_oracle.py, and the golden
// vectors of tests/golden/glue_n256.npz that tests/golden/make_glue_golden.py
// writes from it).
//
// Bound reference code (sph_yamauchi/run): HelmholtzGas::referEquationOfState
// (hdr_hgas.hpp:318-344), SPH::calcBalsaraSwitch (hdr_sph.hpp:79-89),
// HelmholtzGas::calcAlphaDot (hdr_hgas.hpp:750-762), ::calcTimestep
// (hdr_hgas.hpp:477-488), ::calcEnergy (hdr_hgas.hpp:630-634), ::predict and
// ::correct (hdr_hgas.hpp:646-665), SPH::sumAcceleration (hdr_sph.hpp:95-97)
// and calcKernelSupportRadiusMaximum (hdr_util.hpp:489-527).  The global
// reductions around them in main.cpp (calcEnergy's sum, calcTimestep's
// power-of-two step, main.cpp:199-273) sit in a file that also holds main()
// and FDPS's tree set-up, so they are restated in sph_oracle.c only.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>

enum KernelType { CubicSpline = 0, WendlandC2 = 1, WendlandC4 = 2 };  // main.cpp:8

#include "hgas_shim.hpp"
#include "hdr_time.hpp"
#include "hdr_run.hpp"
#include "hdr_dimension.hpp"
#include "hdr_kernel.hpp"
#include "hdr_sph.hpp"
#include "hdr_hgas.hpp"

namespace {

// The particle container calcKernelSupportRadiusMaximum iterates over.
struct Particles {
    HelmholtzGas *p;
    int64_t n;
    int64_t getNumberOfParticleLocal() const { return n; }
    HelmholtzGas &operator[](int64_t i) { return p[i]; }
};

void vec_in(PS::F64vec &v, const double *a, int64_t i) { v = PS::F64vec(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }
void vec_out(const PS::F64vec &v, double *a, int64_t i) {
    a[3 * i] = v.x;
    a[3 * i + 1] = v.y;
    a[3 * i + 2] = v.z;
}

}  // namespace

extern "C" {

void ref_glue_eos(int64_t n, const double *dens, const double *uene, double *pres, double *vsnd) {
    for (int64_t i = 0; i < n; ++i) {
        HelmholtzGas g;
        g.dens = dens[i];
        g.uene = uene[i];
        g.referEquationOfState();
        pres[i] = g.pres;
        vsnd[i] = g.vsnd;
    }
}

void ref_glue_balsara(int64_t n, const double *divv, const double *rotv, const double *vsnd, const double *ksr,
                      double *bswt) {
    for (int64_t i = 0; i < n; ++i) {
        HelmholtzGas g;
        g.divv = divv[i];
        g.rotv = rotv[i];
        g.vsnd = vsnd[i];
        g.ksr = ksr[i];
        g.calcBalsaraSwitch();
        bswt[i] = g.bswt;
    }
}

// alpha derivative only: the reference computes alpha_u's source from an
// EOS minimum energy that its Helmholtz stub (hdr_heos.hpp:21-50) leaves
// unset, so adotu is not bound.
void ref_glue_alpha_dot(int64_t n, const double *divv, const double *alph, const double *vsnd, const double *ksr,
                        double alpha_max, double alpha_min, double *adot) {
    RP::AlphaMaximum = alpha_max;
    RP::AlphaMinimum = alpha_min;
    RP::AlphuMaximum = 0.0;
    RP::AlphuMinimum = 0.0;
    RP::EpsilonOfInternalEnergy = 1.0;
    for (int64_t i = 0; i < n; ++i) {
        HelmholtzGas g;
        g.divv = divv[i];
        g.alph = alph[i];
        g.vsnd = vsnd[i];
        g.ksr = ksr[i];
        g.uene = 1.0;
        g.calcAlphaDot();
        adot[i] = g.adot;
    }
}

// per-particle time step
void ref_glue_timestep(int64_t n, const double *ksr, const double *vsmx, const double *divv, const double *accg1,
                       const double *accg2, double c_dt, double dt_max, double *dt) {
    RP::CoefficientOfTimestep = c_dt;
    RP::MaximumTimestep = dt_max;
    for (int64_t i = 0; i < n; ++i) {
        HelmholtzGas g;
        g.ksr = ksr[i];
        g.vsmx = vsmx[i];
        g.divv = divv[i];
        vec_in(g.accg1, accg1, i);
        vec_in(g.accg2, accg2, i);
        dt[i] = g.calcTimestep();
    }
}

// per-particle energies (their sum, in index order, is main.cpp's calcEnergy)
void ref_glue_energy(int64_t n, const double *mass, const double *vel, const double *uene, const double *pot,
                     double *e) {
    for (int64_t i = 0; i < n; ++i) {
        HelmholtzGas g;
        g.mass = mass[i];
        vec_in(g.vel, vel, i);
        g.uene = uene[i];
        g.pot = pot[i];
        e[i] = g.calcEnergy();
    }
}

// predictor then, with the new derivatives, corrector; in place
void ref_glue_predict(int64_t n, double dt, double *pos, double *vel, const double *acc, double *vel2,
                      double *uene, double *uene2, const double *udot, double *alph, double *alph2,
                      const double *adot, double *alphu, double *alphu2, const double *adotu) {
    for (int64_t i = 0; i < n; ++i) {
        HelmholtzGas g;
        vec_in(g.pos, pos, i);
        vec_in(g.vel, vel, i);
        vec_in(g.acc, acc, i);
        g.uene = uene[i];
        g.udot = udot[i];
        g.alph = alph[i];
        g.adot = adot[i];
        g.alphu = alphu[i];
        g.adotu = adotu[i];
        g.predict(dt);
        vec_out(g.pos, pos, i);
        vec_out(g.vel, vel, i);
        vec_out(g.vel2, vel2, i);
        uene[i] = g.uene;
        uene2[i] = g.uene2;
        alph[i] = g.alph;
        alph2[i] = g.alph2;
        alphu[i] = g.alphu;
        alphu2[i] = g.alphu2;
    }
}

void ref_glue_correct(int64_t n, double dt, double *vel, const double *vel2, const double *acc, double *uene,
                      const double *uene2, const double *udot, double *alph, const double *alph2,
                      const double *adot, double *alphu, const double *alphu2, const double *adotu) {
    for (int64_t i = 0; i < n; ++i) {
        HelmholtzGas g;
        vec_in(g.vel2, vel2, i);
        vec_in(g.acc, acc, i);
        g.uene2 = uene2[i];
        g.udot = udot[i];
        g.alph2 = alph2[i];
        g.adot = adot[i];
        g.alphu2 = alphu2[i];
        g.adotu = adotu[i];
        g.correct(dt);
        vec_out(g.vel, vel, i);
        uene[i] = g.uene;
        alph[i] = g.alph;
        alphu[i] = g.alphu;
    }
}

void ref_glue_sum_acceleration(int64_t n, const double *acch, const double *accg1, const double *accg2,
                               double *acc) {
    for (int64_t i = 0; i < n; ++i) {
        HelmholtzGas g;
        vec_in(g.acch, acch, i);
        vec_in(g.accg1, accg1, i);
        vec_in(g.accg2, accg2, i);
        g.sumAcceleration();
        vec_out(g.acc, acc, i);
    }
}

double ref_glue_ksrmax(int64_t n, const double *mass, const double *pos, const double *vel, const int32_t *istar,
                       const double *dens) {
    RP::FlagBinary = 0;
    HelmholtzGas *p = new HelmholtzGas[n > 0 ? n : 1];
    for (int64_t i = 0; i < n; ++i) {
        p[i].mass = mass[i];
        vec_in(p[i].pos, pos, i);
        vec_in(p[i].vel, vel, i);
        p[i].istar = istar[i];
        p[i].dens = dens[i];
    }
    Particles sys{p, n};
    const double r = calcKernelSupportRadiusMaximum(sys);
    delete[] p;
    return r;
}

}  // extern "C"
