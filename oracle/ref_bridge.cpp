// ref_bridge.cpp — the reference's own CPU functors behind a C ABI.
// TEST INFRASTRUCTURE: compiled by `make -C oracle ref` from the reference
// source tree (REF_DIR, read in place, never copied) into oracle/_ref/.  It is
// the oracle the C restatement in sph_oracle.c is checked against; the
// golden vectors under tests/golden/ are its outputs.
//
// Included reference headers (sph_yamauchi/run): hdr_run.hpp,
// hdr_dimension.hpp, hdr_kernel.hpp, hdr_sph.hpp, hdr_density.hpp,
// hdr_hydro.hpp, hdr_gravity.hpp, plus vector_x86.hpp for the AVX2 build.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#ifdef _OPENMP
#include <omp.h>
#endif

enum KernelType { CubicSpline = 0, WendlandC2 = 1, WendlandC4 = 2 };  // main.cpp:8

#include "particle_simulator.hpp"
#include "hdr_run.hpp"
#ifdef USE_INTRINSICS
#include "vector_x86.hpp"
#endif
#include "hdr_dimension.hpp"
#include "hdr_kernel.hpp"
#include "hdr_sph.hpp"

// hdr_hydro.hpp / hdr_gravity.hpp name CodeUnit::GravityConstantInThisUnit in
// their write-back methods; the bridge never calls those, the value is moot.
namespace CodeUnit {
PS::F64 GravityConstantInThisUnit = 1.0;
}

// hdr_gravity.hpp defines copyFromForce/copyFromFP for these two classes
// (hdr_msls.hpp / hdr_bhns.hpp need the full EOS stack); declarations only.
class MassLess : public SPH {
public:
    void copyFromForce(const Gravity &gravity);
};
class BlackHoleNeutronStar : public SPH {
public:
    PS::F64 eps;
    void copyFromForce(const Gravity &gravity);
};

#include "hdr_density.hpp"
#include "hdr_hydro.hpp"
#include "hdr_gravity.hpp"

#include "../include/sph_gb300.h"

static_assert(sizeof(DensityEPI) == sizeof(sph_DensityEPI), "DensityEPI layout");
static_assert(sizeof(DensityEPJ) == sizeof(sph_DensityEPJ), "DensityEPJ layout");
static_assert(sizeof(Density) == sizeof(sph_Density), "Density layout");
static_assert(sizeof(HydroEPI) == sizeof(sph_HydroEPI), "HydroEPI layout");
static_assert(sizeof(HydroEPJ) == sizeof(sph_HydroEPJ), "HydroEPJ layout");
static_assert(sizeof(Hydro) == sizeof(sph_Hydro), "Hydro layout");
static_assert(sizeof(GravityEPI) == sizeof(sph_GravityEPI), "GravityEPI layout");
static_assert(sizeof(GravityEPJ) == sizeof(sph_GravityEPJ), "GravityEPJ layout");
static_assert(sizeof(PS::GravitySPJ) == sizeof(sph_GravitySPJ), "GravitySPJ layout");
static_assert(sizeof(Gravity) == sizeof(sph_Gravity), "Gravity layout");

static void setup(double ksr_max) {
    RP::NumberOfDimension = 3;  // set by initializeSimulation, hdr_hgas.hpp:1253-1257
    RP::KernelSupportRadiusMaximum = (ksr_max > 0.0) ? ksr_max : 1e300;
}

template <class Dst, class Src>
static void copy_in(Dst *dst, const Src *src, int n) {
    for (int k = 0; k < n; ++k) std::memcpy(&dst[k], &src[k], sizeof(Src));
}

extern "C" {

// SmoothingKernel::eta is a compile-time constant (1.6) in the reference.
double ref_eta(void) { return SK::eta; }

void ref_calc_density(const sph_DensityEPI *epi, int ni, const sph_DensityEPJ *epj, int nj,
                      sph_Density *out, double ksr_max) {
    setup(ksr_max);
    DensityEPI *ri = new DensityEPI[ni > 0 ? ni : 1];
    DensityEPJ *rj = new DensityEPJ[nj > 0 ? nj : 1];
    Density *rf = new Density[ni > 0 ? ni : 1];
    copy_in(ri, epi, ni);
    copy_in(rj, epj, nj);
    for (int k = 0; k < ni; ++k) rf[k].clear();
    calcDensity()(ri, ni, rj, nj, rf);
    for (int k = 0; k < ni; ++k) std::memcpy(&out[k], &rf[k], sizeof(sph_Density));
    delete[] ri;
    delete[] rj;
    delete[] rf;
}

void ref_calc_hydro(const sph_HydroEPI *epi, int ni, const sph_HydroEPJ *epj, int nj,
                    sph_Hydro *out) {
    setup(0.0);
    HydroEPI *ri = new HydroEPI[ni > 0 ? ni : 1];
    HydroEPJ *rj = new HydroEPJ[nj > 0 ? nj : 1];
    Hydro *rf = new Hydro[ni > 0 ? ni : 1];
    copy_in(ri, epi, ni);
    copy_in(rj, epj, nj);
    for (int k = 0; k < ni; ++k) rf[k].clear();
    calcHydro()(ri, ni, rj, nj, rf);
    for (int k = 0; k < ni; ++k) std::memcpy(&out[k], &rf[k], sizeof(sph_Hydro));
    delete[] ri;
    delete[] rj;
    delete[] rf;
}

// Accumulates into out, like the reference functor.
void ref_calc_gravity_ep(const sph_GravityEPI *epi, int ni, const sph_GravityEPJ *epj, int nj,
                         sph_Gravity *out) {
    setup(0.0);
    GravityEPI *ri = new GravityEPI[ni > 0 ? ni : 1];
    GravityEPJ *rj = new GravityEPJ[nj > 0 ? nj : 1];
    Gravity *rf = new Gravity[ni > 0 ? ni : 1];
    copy_in(ri, epi, ni);
    copy_in(rj, epj, nj);
    for (int k = 0; k < ni; ++k) std::memcpy(&rf[k], &out[k], sizeof(sph_Gravity));
    calcGravity<GravityEPJ>()(ri, ni, rj, nj, rf);
    for (int k = 0; k < ni; ++k) std::memcpy(&out[k], &rf[k], sizeof(sph_Gravity));
    delete[] ri;
    delete[] rj;
    delete[] rf;
}

void ref_calc_gravity_sp(const sph_GravityEPI *epi, int ni, const sph_GravitySPJ *spj, int nj,
                         sph_Gravity *out) {
    setup(0.0);
    GravityEPI *ri = new GravityEPI[ni > 0 ? ni : 1];
    PS::GravitySPJ *rj = new PS::GravitySPJ[nj > 0 ? nj : 1];
    Gravity *rf = new Gravity[ni > 0 ? ni : 1];
    copy_in(ri, epi, ni);
    copy_in(rj, spj, nj);
    for (int k = 0; k < ni; ++k) std::memcpy(&rf[k], &out[k], sizeof(sph_Gravity));
    calcGravity<PS::GravitySPJ>()(ri, ni, rj, nj, rf);
    for (int k = 0; k < ni; ++k) std::memcpy(&out[k], &rf[k], sizeof(sph_Gravity));
    delete[] ri;
    delete[] rj;
    delete[] rf;
}

// Walk-batched variants with OpenMP over walks: the CPU baseline's threading
// (FDPS runs the functors per walk from OpenMP threads, Makefile:89-91).
int ref_density_walks(int n_walk, const int64_t *i_off, const int64_t *j_off,
                      const sph_DensityEPI *epi, const sph_DensityEPJ *epj, sph_Density *out,
                      double ksr_max, int nthreads) {
    setup(ksr_max);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    static_assert(sizeof(DensityEPI) == sizeof(sph_DensityEPI), "");
#pragma omp parallel for schedule(dynamic, 1)
    for (int w = 0; w < n_walk; ++w) {
        const int ni = (int)(i_off[w + 1] - i_off[w]);
        const int nj = (int)(j_off[w + 1] - j_off[w]);
        calcDensity()(reinterpret_cast<const DensityEPI *>(epi + i_off[w]), ni,
                      reinterpret_cast<const DensityEPJ *>(epj + j_off[w]), nj,
                      reinterpret_cast<Density *>(out + i_off[w]));
    }
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int ref_hydro_walks(int n_walk, const int64_t *i_off, const int64_t *j_off,
                    const sph_HydroEPI *epi, const sph_HydroEPJ *epj, sph_Hydro *out,
                    int nthreads) {
    setup(0.0);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int w = 0; w < n_walk; ++w) {
        const int ni = (int)(i_off[w + 1] - i_off[w]);
        const int nj = (int)(j_off[w + 1] - j_off[w]);
        calcHydro()(reinterpret_cast<const HydroEPI *>(epi + i_off[w]), ni,
                    reinterpret_cast<const HydroEPJ *>(epj + j_off[w]), nj,
                    reinterpret_cast<Hydro *>(out + i_off[w]));
    }
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int ref_gravity_walks(int n_walk, const int64_t *i_off, const int64_t *j_off,
                      const sph_GravityEPI *epi, const sph_GravityEPJ *epj, sph_Gravity *out,
                      int nthreads) {
    setup(0.0);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int w = 0; w < n_walk; ++w) {
        const int ni = (int)(i_off[w + 1] - i_off[w]);
        const int nj = (int)(j_off[w + 1] - j_off[w]);
        Gravity *f = reinterpret_cast<Gravity *>(out + i_off[w]);
        for (int k = 0; k < ni; ++k) f[k].clear();
        calcGravity<GravityEPJ>()(reinterpret_cast<const GravityEPI *>(epi + i_off[w]), ni,
                                  reinterpret_cast<const GravityEPJ *>(epj + j_off[w]), nj, f);
    }
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
