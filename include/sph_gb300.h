/*
 * sph_gb300.h — C ABI of the GB300 SPH interaction engine.
 *
 * The engine computes the three per-step pair interactions of the FDPS-based
 * SPH stellar-collision code yamauchi1132/Research_Codes (sph_yamauchi/run):
 *   - the density sum with the fixed 3-pass smoothing-length iteration and the
 *     grad-h / div v / |rot v| pass            (hdr_density.hpp:246-366)
 *   - the hydro force: pressure gradient, Balsara-switched artificial
 *     viscosity, du/dt, conduction signal, v_sig max and the gravity
 *     softening correction                     (hdr_hydro.hpp:312-424)
 *   - the softened tree-gravity sum over particles and monopoles
 *                                              (hdr_gravity.hpp:286-342)
 * on sm_103a CUDA cores.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (SPH_OK == 0).  Structs named sph_<Name> reproduce the reference's FDPS
 * particle/force classes byte for byte (offsets are asserted in the library
 * and reported by sph_abi_layout()), so arrays built for the reference's
 * functors can be passed unchanged.
 *
 * Threading: a context owns one CUDA stream and its device buffers; calls on
 * one context must not overlap.  Different contexts may be used from
 * different host threads.
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stdint.h>
#include <stddef.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes.  The reference has no error channel (void functors,
 * Dispatch/Retrieve return 0, limits are assert()s: hdr_densityGPU.cu:503,
 * 521-522); these replace the asserts and never abort the process.          */
enum sph_status {
    SPH_OK                   = 0,
    SPH_ERR_INVALID_ARGUMENT = 1,  /* null pointer, negative count, bad enum  */
    SPH_ERR_CAPACITY         = 2,  /* walk / i / j count beyond the capacity  */
    SPH_ERR_CUDA             = 3,  /* a CUDA runtime call failed              */
    SPH_ERR_NONFINITE        = 4,  /* NaN/Inf found in an output              */
    SPH_ERR_NOT_CONVERGED    = 5,  /* search-radius expansion hit its cap     */
    SPH_ERR_STATE            = 6,  /* e.g. Retrieve without a Dispatch        */
    SPH_ERR_NO_DEVICE        = 7   /* no CUDA device / unsupported device     */
};

/* Arithmetic of the pair kernels. */
enum sph_precision {
    /* FP32 pair arithmetic on positions/velocities taken relative to each
     * i-group's centre, compensated (Kahan) accumulation; per-particle
     * scalars (h update, Omega, write-back) in FP64.                        */
    SPH_PREC_FP32C = 0,
    /* Plain FP64 pair arithmetic on global coordinates. */
    SPH_PREC_FP64  = 1
};

/* ------------------------------------------------------------------------ */
/* Reference POD layouts (FDPS EPI / EPJ / SPJ / Force classes).             */

/* DensityEPI, hdr_density.hpp:33-58 (80 bytes). */
typedef struct sph_DensityEPI {
    int32_t id;
    double  mass;
    double  pos[3];
    double  vel[3];
    double  ksr;   /* kernel support radius h used as the first guess */
    double  rs;    /* search radius the j-list was built with          */
} sph_DensityEPI;

/* DensityEPJ, hdr_density.hpp:60-78 (64 bytes). */
typedef struct sph_DensityEPJ {
    int32_t id;
    double  mass;
    double  pos[3];
    double  vel[3];
} sph_DensityEPJ;

/* Density (force), hdr_density.hpp:4-22 (56 bytes). */
typedef struct sph_Density {
    double  dens;
    double  divv;
    double  rotv;
    double  grdh;  /* Omega = 1 / (1 + h/(3 rho) d rho/dh) */
    double  ksr;
    int64_t np;    /* neighbour count of the last h pass */
    bool    itr;   /* final h exceeds the search radius rs */
} sph_Density;

/* HydroEPI, hdr_hydro.hpp:28-75 (144 bytes). */
typedef struct sph_HydroEPI {
    int64_t id;
    double  pos[3];
    double  vel[3];
    double  ksr;
    double  hinv;
    double  pres;
    double  presc;  /* P * Omega / rho^2 */
    double  bswt;   /* 0.5 * Balsara switch */
    double  dens;
    double  vsnd;
    double  alph;
    double  alphu;
    double  thrm;   /* max(u - umin, 0) */
    double  eta;    /* gravity-softening correction coefficient */
} sph_HydroEPI;

/* HydroEPJ, hdr_hydro.hpp:77-126 (152 bytes). */
typedef struct sph_HydroEPJ {
    int64_t id;
    double  mass;
    double  pos[3];
    double  vel[3];
    double  ksr;
    double  hinv;
    double  pres;
    double  presc;
    double  bswt;
    double  dens;
    double  vsnd;
    double  alph;
    double  alphu;
    double  thrm;
    double  eta;
} sph_HydroEPJ;

/* Hydro (force), hdr_hydro.hpp:3-17 (72 bytes). */
typedef struct sph_Hydro {
    double acch[3];
    double accg[3];
    double udot;
    double vsmx;
    double diffu;
} sph_Hydro;

/* GravityEPI, hdr_gravity.hpp:130-155 (32 bytes). */
typedef struct sph_GravityEPI {
    double pos[3];
    double eps2;
} sph_GravityEPI;

/* GravityEPJ, hdr_gravity.hpp:157-192 (40 bytes). */
typedef struct sph_GravityEPJ {
    double mass;
    double pos[3];
    double eps2;
} sph_GravityEPJ;

/* PS::GravitySPJ, hdr_gravity.hpp:63-91 (40 bytes). */
typedef struct sph_GravitySPJ {
    double mass;
    double pos[3];
    double eps2;
} sph_GravitySPJ;

/* Gravity (force), hdr_gravity.hpp:95-105 (40 bytes). */
typedef struct sph_Gravity {
    double acc[3];
    double pot;
    double eta;
} sph_Gravity;

/* ------------------------------------------------------------------------ */
/* Context.                                                                  */

typedef struct sph_params {
    int32_t device;      /* CUDA device ordinal                                */
    int32_t precision;   /* enum sph_precision                                 */
    double  eta;         /* h = eta * ksrh * (m/rho)^(1/3); reference: 1.6
                            (hdr_kernel.hpp:218)                              */
    double  ksr_max;     /* KernelSupportRadiusMaximum clamp of h; 0 disables
                            the clamp, matching ksrmax=+inf                   */
    int32_t max_walks;   /* walks per dispatch (reference N_WALK_LIMIT=1000,
                            use_gpu.hpp:20-26)                                */
    int64_t max_i;       /* i-particles per dispatch (NI_LIMIT = 1e6)          */
    int64_t max_j;       /* j entries per dispatch   (NJ_LIMIT = 1e7)          */
    int32_t check_finite;/* non-zero: scan outputs, return SPH_ERR_NONFINITE   */
} sph_params;

typedef struct sph_context sph_context;

/* Fills *p with defaults: device 0, FP32C, eta 1.6, no clamp, the reference's
 * buffer limits, finite check on. */
void sph_params_default(sph_params *p);

/* Creates a context on p->device with one stream and buffers sized by the
 * capacities in *p.  No counterpart call in the reference: its buffers are
 * file-static and allocated on the first Dispatch (hdr_densityGPU.cu:486-511). */
int  sph_context_create(const sph_params *p, sph_context **out);
int  sph_context_destroy(sph_context *ctx);

/* Updates eta / ksr_max / precision between calls (the reference re-uploads
 * ksrmax to constant memory on every dispatch, hdr_densityGPU.cu:581). */
int  sph_context_set_eta(sph_context *ctx, double eta);
int  sph_context_set_ksr_max(sph_context *ctx, double ksr_max);
int  sph_context_set_precision(sph_context *ctx, int32_t precision);

/* The context's CUDA stream (a cudaStream_t) for callers that order their
 * own work or record events around the engine's calls. */
int  sph_context_stream(const sph_context *ctx, void **stream);

/* Measures the FP32 FMA throughput of the context's device (TFLOP/s) with a
 * register-resident FMA loop on every SM: the denominator of the pair
 * kernels' roofline. */
int  sph_probe_fp32_peak(sph_context *ctx, double *tflops);

/* Human-readable text for a status code (static storage). */
const char *sph_status_string(int status);
/* Detail text of the last failure on this context (copied into buf). */
int  sph_context_last_error(const sph_context *ctx, char *buf, size_t n);

/* ------------------------------------------------------------------------ */
/* Single-group functors: the FDPS interaction-functor signature
 *   operator()(const EPI *epi, S32 n_i, const EPJ *epj, S32 n_j, Force *f)
 * with the context in front.  Synchronous.                                  */

/* calcDensity::operator(), hdr_density.hpp:248-252.  Assigns force[0..n_i). */
int sph_calc_density(sph_context *ctx,
                     const sph_DensityEPI *epi, int32_t n_i,
                     const sph_DensityEPJ *epj, int32_t n_j,
                     sph_Density *force);

/* calcHydro::operator(), hdr_hydro.hpp:314-318.  Assigns force[0..n_i). */
int sph_calc_hydro(sph_context *ctx,
                   const sph_HydroEPI *epi, int32_t n_i,
                   const sph_HydroEPJ *epj, int32_t n_j,
                   sph_Hydro *force);

/* calcGravity<GravityEPJ>::operator(), hdr_gravity.hpp:289-293.
 * ACCUMULATES into force[0..n_i) like the reference; clear it first. */
int sph_calc_gravity_ep(sph_context *ctx,
                        const sph_GravityEPI *epi, int32_t n_i,
                        const sph_GravityEPJ *epj, int32_t n_j,
                        sph_Gravity *force);

/* calcGravity<PS::GravitySPJ>::operator() (the same template, called for the
 * superparticles, hdr_gravity.hpp:400-402).  Accumulates. */
int sph_calc_gravity_sp(sph_context *ctx,
                        const sph_GravityEPI *epi, int32_t n_i,
                        const sph_GravitySPJ *spj, int32_t n_j,
                        sph_Gravity *force);

/* Allocation-free variant of sph_calc_gravity_ep for callers that cannot
 * allocate device memory: host code that must not synchronise the device (an
 * allocation can), such as a hook another library calls on its hot path —
 * not a CUDA stream callback or cudaLaunchHostFunc function, where no CUDA
 * call is allowed —, runtimes that own all device memory through a fixed
 * arena, loops that cannot afford an allocation's latency or failure in
 * mid-run.  No counterpart in the reference.
 *
 * epi, epj and force are DEVICE pointers owned by the caller; the work is
 * queued on `stream` (a cudaStream_t, NULL = default stream) and the call
 * returns without waiting.  FP32C arithmetic; forces ACCUMULATE like the
 * reference functor.  Scratch lives in one file-scope __device__ array of the
 * library (~2.4 MB, held by every GPU that loads the library until the process
 * exits), which bounds a call to n_i <= SPH_NOALLOC_MAX_I and
 * n_j <= SPH_NOALLOC_MAX_J (larger calls return SPH_ERR_CAPACITY).  Every call
 * looks up the array's device address with the caller's device current
 * (cudaGetSymbolAddress); the first call on a device may load the library's
 * module, which can allocate and synchronise: make it during set-up, before
 * any stream capture.  A CUDA error pending from the caller's earlier work is
 * returned as SPH_ERR_CUDA and left for the caller to read.  All calls share
 * the array; calls that overlap on the GPU race and must be serialised by the
 * caller. */
#define SPH_NOALLOC_MAX_I 4096
#define SPH_NOALLOC_MAX_J 65536
int sph_calc_gravity_ep_noalloc(const sph_GravityEPI *epi, int32_t n_i,
                                const sph_GravityEPJ *epj, int32_t n_j,
                                sph_Gravity *force, void *stream);

/* ------------------------------------------------------------------------ */
/* Batched multiwalk pairs (use_gpu.hpp:28-64).  Dispatch copies the walks to
 * the device and launches; it returns before the kernel finishes.  Retrieve
 * waits and writes force[w][0..n_i[w]).  Density/Hydro/Gravity results are
 * ASSIGNED (the reference's Retrieve* assign, hdr_gravityGPU.cu:484-489).
 * tag is accepted for signature parity; one dispatch may be outstanding per
 * context and interaction kind. */

/* DispatchKernel_Dens / RetrieveKernel_Dens, hdr_densityGPU.cu:496-621 */
int sph_dispatch_density(sph_context *ctx, int32_t tag, int32_t n_walk,
                         const sph_DensityEPI **epi, const int32_t *n_epi,
                         const sph_DensityEPJ **epj, const int32_t *n_epj);
int sph_retrieve_density(sph_context *ctx, int32_t tag, int32_t n_walk,
                         const int32_t *n_i, sph_Density **force);

/* DispatchKernel_HydroForce / RetrieveKernel_HydroForce,
 * hdr_hydroGPU.cu:371-507 */
int sph_dispatch_hydro(sph_context *ctx, int32_t tag, int32_t n_walk,
                       const sph_HydroEPI **epi, const int32_t *n_epi,
                       const sph_HydroEPJ **epj, const int32_t *n_epj);
int sph_retrieve_hydro(sph_context *ctx, int32_t tag, int32_t n_walk,
                       const int32_t *n_i, sph_Hydro **force);

/* DispatchKernel_Gravity / RetrieveKernel_Gravity,
 * hdr_gravityGPU.cu:383-495.  The j-list of walk w is its EPJ followed by its
 * SPJ, as the reference appends them (hdr_gravityGPU.cu:445-453). */
int sph_dispatch_gravity(sph_context *ctx, int32_t tag, int32_t n_walk,
                         const sph_GravityEPI **epi, const int32_t *n_epi,
                         const sph_GravityEPJ **epj, const int32_t *n_epj,
                         const sph_GravitySPJ **spj, const int32_t *n_spj);
int sph_retrieve_gravity(sph_context *ctx, int32_t tag, int32_t n_walk,
                         const int32_t *n_i, sph_Gravity **force);

/* ------------------------------------------------------------------------ */
/* Device-resident particle system: the whole calcSPHKernel step on the GPU.
 *
 * Replaces the reference's per-step driver around the functors:
 *   loopSimulation (hdr_hgas.hpp:1469-1542): calcTimestep (main.cpp:242-273),
 *   predict (hdr_hgas.hpp:646-657), calcSPHKernel (main.cpp:300-358) =
 *   calcDensityKernel (hdr_density.hpp:372-415) -> EOS (hdr_hgas.hpp:318-344)
 *   -> Balsara (hdr_sph.hpp:79-89) -> gravity (hdr_gravity.hpp:351-423) ->
 *   hydro -> sumAcceleration / calcAlphaDot / ksrmax (hdr_util.hpp:489-527),
 *   correct (hdr_hgas.hpp:659-665).
 * The tree, the i-groups and the interaction lists that FDPS builds for the
 * reference are built on the GPU (Morton-sorted binary radix tree).  Particle
 * state stays in HBM in Morton order between calls; uploads and downloads
 * use the caller's (upload) order.  A step can be captured as a CUDA graph.  */

typedef struct sph_system sph_system;

typedef struct sph_system_params {
    int32_t n_group;     /* max i-particles per walk (FDPS n_group, main.cpp:380: 256) */
    int32_t n_leaf;      /* particle bucket of the tree walk (FDPS n_leaf: 8)           */
    double  theta;       /* gravity opening angle (main.cpp:394: 0.5)                   */
    double  G;           /* gravitational constant in code units (hdr_heos.hpp:102)     */
    double  c_dt;        /* CoefficientOfTimestep (0.1)                                 */
    double  dt_max;      /* MaximumTimestep (hdr_hgas.hpp:1240: 10); finite, >= dt_min   */
    double  dt_min;      /* MinimumTimestep (1e-16); > 0, else INVALID_ARGUMENT         */
    double  alpha_max, alpha_min, alphu_max, alphu_min;  /* .head run parameters       */
    int32_t ksr_max_mode;/* 0: the context's fixed ksr_max; 1: the reference rule —
                            star-centre separation at start (hdr_hgas.hpp:1335), then
                            the density-weighted rms radius about star 0's centre of
                            mass after every force evaluation (hdr_util.hpp:489-527)   */
    int32_t max_density_iterations; /* cap on search-radius expansions              */
    int32_t use_graph;   /* capture sph_system_step's body as a CUDA graph              */
    int32_t quadrupole;  /* 1: tree nodes accepted by the gravity walk act with their
                            mass and traceless quadrupole (no counterpart in the
                            reference, whose SPJ is a monopole, hdr_gravity.hpp:6-91);
                            0: monopole, as the reference                             */
    int32_t item_split_nj; /* density / hydro walks whose list is longer than this are
                            cut into work items of 16, 8 or 4 i-particles (<= 0: 4096) */
    int32_t heavy_classes; /* work items of this many most expensive cost classes run
                            first, the rest in walk order (< 0: 2)                      */
    float   density_list_slack; /* radius of the density kernel's per-lane neighbour
                            lists over each particle's first-pass h (default 1.03): the
                            first pass writes them, the later passes and the gradient
                            pass read them while h stays within it; <= 0 or NaN: no
                            lists, every pass streams the walk's j-list; above 2 the
                            create / set_params calls fail with INVALID_ARGUMENT       */
    int32_t hydro_signal_skip; /* 1 (default): hydro tiles of 32 j-entries whose
                            signal-velocity terms provably cannot raise any i-particle's
                            maximum skip those terms (results unchanged bit for bit);
                            0: every term is evaluated                                 */
    int32_t gravity_jtile; /* FP32C gravity: list entries a warp stages in shared
                            memory and sums per pass, 32 (default) or 64; other values
                            fail with INVALID_ARGUMENT                                 */
} sph_system_params;

/* Fields for sph_system_download / sph_system_download_sorted. */
enum sph_field {
    SPH_F_POS = 0, SPH_F_VEL = 1, SPH_F_ACC = 2, SPH_F_ACCH = 3, SPH_F_ACCG1 = 4,
    SPH_F_ACCG2 = 5,                                  /* 3 doubles per particle */
    SPH_F_MASS = 10, SPH_F_DENS = 11, SPH_F_PRES = 12, SPH_F_VSND = 13, SPH_F_KSR = 14,
    SPH_F_DIVV = 15, SPH_F_ROTV = 16, SPH_F_BSWT = 17, SPH_F_GRDH = 18, SPH_F_UENE = 19,
    SPH_F_UDOT = 20, SPH_F_ALPH = 21, SPH_F_ALPHU = 22, SPH_F_POT = 23, SPH_F_ETA = 24,
    SPH_F_VSMX = 25, SPH_F_DIFFU = 26, SPH_F_NP = 27, SPH_F_ADOT = 28, SPH_F_ADOTU = 29,
    SPH_F_ID = 30, SPH_F_ISTAR = 31                    /* 1 double per particle */
};

typedef struct sph_system_stats {
    double  time, dt, ksr_max;
    double  e_kin, e_thm, e_pot, e_tot;   /* FP64 sums, sum m(v^2/2), m u, m pot/2 */
    int64_t n_groups;
    int64_t density_iterations;           /* walks of the last density evaluation */
    int64_t pairs_density;                /* sum over walks of n_i * n_j, all
                                             search-radius walks                  */
    int64_t pairs_density_first;          /* the first density walk alone         */
    int64_t pairs_hydro;
    int64_t pairs_gravity;                /* particles + monopoles                */
    int64_t list_density, list_hydro, list_gravity;  /* list entries            */
    int64_t steps;
    int64_t density_rechecked;            /* FP32C results re-evaluated in FP64
                                             because h fell within 4e-6 of rs    */
    int64_t evals_density_first;          /* pair evaluations the density kernel
                                             performed in the first walk, three
                                             density passes (j beyond every i's
                                             support dropped before the loop)    */
    int64_t evals_density_grad;           /* the same for its gradient pass       */
    int64_t evals_hydro_near;             /* hydro pairs evaluated in full        */
    int64_t evals_hydro_far;              /* hydro pairs beyond both supports,
                                             signal velocity only                */
    int64_t density_list_passes;          /* first walk: work-item passes after
                                             the first (second, third, gradient)
                                             served from neighbour lists         */
    int64_t density_sweep_passes;         /* ... that swept the walk's j-list     */
    int64_t hydro_sv_tiles_skipped;       /* hydro 32-entry tiles whose signal-
                                             velocity terms provably could not
                                             raise any lane's maximum (skipped)  */
    int64_t hydro_sv_tiles;               /* hydro tiles tested                   */
    int64_t hydro_pairs_marked;           /* hydro pairs inside either support
                                             (the terms evaluated in full)       */
    int64_t hydro_pair_slots;             /* lane slots the loops over them took
                                             (32 x the largest per-lane count of
                                             each tile); marked / slots is the
                                             lane utilisation of those loops     */
    int64_t hydro_rows_overflowed;        /* FP32C: particles with more marked
                                             pairs than a list row holds (summed
                                             over the walk's whole list instead) */
    int32_t last_status;
} sph_system_stats;

void sph_system_params_default(sph_system_params *p);

/* Changes the run parameters of an existing system (the next evaluation
 * re-captures its graphs): n_group, n_leaf, theta, the time-step and
 * viscosity parameters, item_split_nj and heavy_classes; quadrupole may only
 * be switched on if the system was created with it. */
int sph_system_set_params(sph_system *sys, const sph_system_params *p);

/* Allocates a system of n particles on the context's device. */
int sph_system_create(sph_context *ctx, int64_t n, const sph_system_params *p,
                      sph_system **out);
int sph_system_destroy(sph_system *sys);

/* Host -> device copy of the particle state (arrays of n, pos/vel n*3).
 * alph / alphu / istar may be null (1.0 / 0.0 / 0).  Resets time to t0. */
int sph_system_upload(sph_system *sys, double t0, const int64_t *id, const int32_t *istar,
                      const double *mass, const double *pos, const double *vel,
                      const double *uene, const double *ksr, const double *alph,
                      const double *alphu);

/* calcSPHKernel on the current state (the force evaluation of
 * startSimulation, hdr_hgas.hpp:1378): density, EOS, gravity, hydro,
 * accelerations, alpha derivatives, ksrmax.  Fills the stats' pair counts. */
int sph_system_compute_forces(sph_system *sys);

/* n_steps iterations of the reference's loop body: time step, predict,
 * calcSPHKernel, correct. */
int sph_system_step(sph_system *sys, int32_t n_steps);

/* Switches CUDA-graph replay of compute_forces / step on or off (off: every
 * call runs eagerly, e.g. for per-phase event timings). */
int sph_system_set_graph(sph_system *sys, int32_t use_graph);

/* Device -> host copy of one field in upload order (3 or 1 doubles each). */
int sph_system_download(sph_system *sys, int32_t field, double *out);
/* The same in the system's current (Morton) order, matching the lists. */
int sph_system_download_sorted(sph_system *sys, int32_t field, double *out);

int sph_system_get_stats(sph_system *sys, sph_system_stats *out);

/* Host -> device copy of one per-particle field in upload order, for
 * restarting from a checkpoint (the reference's readHexa restores the whole
 * particle state, hdr_hgas.hpp:198-284, and continues without a new force
 * evaluation, hdr_hgas.hpp:1383-1412).  Any field of sph_field except
 * SPH_F_POS, SPH_F_VEL, SPH_F_MASS, SPH_F_NP, SPH_F_ID and SPH_F_ISTAR, which
 * sph_system_upload sets. */
int sph_system_set_field(sph_system *sys, int32_t field, const double *data);

/* Run clock and the run parameters derived from the state: time, current
 * time step, kernel-support-radius cap (ksrmax) and the internal-energy floor
 * epsu (the reference keeps them in the checkpoint header,
 * hdr_hgas.hpp:890-926).  set: a negative value leaves an entry unchanged. */
int sph_system_get_clock(sph_system *sys, double *time, double *dt, double *ksr_max, double *eps_u);
int sph_system_set_clock(sph_system *sys, double time, double dt, double ksr_max, double eps_u);

/* Derivative of the step (no counterpart in the reference, which has no
 * gradients).  sph_system_predict runs the leapfrog predictor alone
 * (hdr_hgas.hpp:646-657) with the clock's dt; followed by
 * sph_system_compute_forces it repeats the force evaluation of a step from
 * that step's starting state.  sph_system_adjoint_forces is the
 * vector-Jacobian product of the last force evaluation, with the lists, tree
 * and dt of that evaluation held fixed:
 *   seed (upload order, 8n doubles): dL/d of the outputs acc (3n), udot (n),
 *        adot (n), ksr (n, the final h), pot (n), dens (n)
 *   grad (upload order, 9n doubles): dL/d of the inputs position (3n),
 *        velocity (3n), uene (n), alph (n), and the first guess of h (n).
 * It needs monopole gravity, alphu_max = alphu_min = 0, no clamp of h
 * (context ksr_max 0 and ksr_max_mode 0) and an evaluation with a single
 * density walk; otherwise SPH_ERR_STATE.  FP64 arithmetic, either precision
 * of the forward evaluation. */
int sph_system_predict(sph_system *sys);
int sph_system_adjoint_forces(sph_system *sys, const double *seed, double *grad);

/* Interaction lists of the last force evaluation (kind 0 density — the first
 * walk, which covers every group —, 1 hydro, 2 gravity, 3 the last density
 * re-walk of the search-radius loop, calcDensityKernel hdr_density.hpp:
 * 372-415), in Morton order: walk w has i-particles [i_first[w], i_first[w]
 * + i_count[w]) and list entries j_idx[j_off[w] .. j_off[w+1]); for gravity
 * an entry >= n is tree node entry - n (see sph_system_get_nodes); a re-walk
 * evaluates only the particles of its groups that were still iterating, with
 * their grown search radius.  Call with null arrays to get *n_walk and
 * *n_entries first. */
int sph_system_get_lists(sph_system *sys, int32_t kind, int32_t *n_walk, int64_t *n_entries,
                         int32_t *i_first, int32_t *i_count, int64_t *j_off, int32_t *j_idx);

/* Device time (ms) of the phases of the most recent force evaluation,
 * from CUDA events recorded on the context's stream (also inside a captured
 * step): [0] tree + groups, [1] density incl. lists and all walks,
 * [2] density pair kernel of the first walk, [3] gravity lists,
 * [4] gravity pair kernel, [5] hydro prep + lists, [6] hydro pair kernels,
 * [7] the whole force evaluation, [8] and [9] the two parts of [6] (FP32C:
 * the signal-velocity / marking kernel and the double-float pass over the
 * marked pairs; FP64: the pair kernel and nothing).  Returns the number of
 * values written, or minus a status code.  Eager evaluations record the
 * events directly; captured graphs (force evaluation and step) hold them as
 * external event-record nodes, so the values after a graph replay are that
 * replay's.  [3] runs on a second stream in captured graphs, overlapping
 * [1]. */
int sph_system_phase_times(sph_system *sys, float *ms, int32_t n);

/* Kernel launches per replay of the captured graph: step = 1 for the
 * sph_system_step graph, 0 for the sph_system_compute_forces graph: its
 * kernel nodes plus, for the density re-walks (a conditional while-node of
 * the graph that runs while particles still iterate), the loop body's kernel
 * nodes times the re-walks of the last evaluation.  SPH_ERR_STATE when that
 * graph has not been captured. */
int sph_system_graph_kernels(sph_system *sys, int32_t step, int64_t *kernels);

/* ---- analysis of the current state on the device (the reference's
 * post-processing scripts).  star < 0: all particles, else those with
 * istar == star. */
/* Density-weighted centre and velocity, analysis/common.py:71-90:
 * out = (x, y, z, vx, vy, vz, sum of densities). */
int sph_system_center_of_gravity(sph_system *sys, int32_t star, double *out);
/* Bound and unbound mass (out[0], out[1]): unbound when
 * |v - vel_ref|^2 / 2 + pot + u > 0, analysis/unbound_mass/unbound_mass.py:10-27. */
int sph_system_bound_mass(sph_system *sys, int32_t star, const double *vel_ref, double *out);
/* Mass within `radius` of `center`, energy_check/energy_check.py:50-68. */
int sph_system_mass_within(sph_system *sys, int32_t star, const double *center, double radius, double *out);
/* Distances of the particles of the set from `center`, sorted ascending on
 * the device, with their masses (arrays of n; the first *count are set), the
 * input of Lagrange radii, analysis/lagrange_radius/lagrange_radius.py:25-47. */
int sph_system_radii_sorted(sph_system *sys, int32_t star, const double *center, double *r, double *m,
                            int64_t *count);

/* Monopoles of the 2n-1 tree nodes: mom[4*k..] = (x, y, z, mass), eps2[k]. */
int sph_system_get_nodes(sph_system *sys, double *mom, double *eps2);

/* ------------------------------------------------------------------------ */
/* Text encodings of the reference's particle files (host only, no device).
 * Rows of n particles: "id istar" then ncol values of cols (row-major n x
 * ncol).  Each returns the number of bytes the text needs (out may be null)
 * and writes it when out holds cap >= that many bytes; minus a status code
 * on bad arguments. */
/* Checkpoint rows: values as the hexadecimal image of their FP64 bits
 * ("%6lld %2lld %llx ..."), HelmholtzGas::writeHexa, hdr_hgas.hpp:286-316. */
int64_t sph_format_hexa_rows(int64_t n, const int64_t *id, const int64_t *istar, int32_t ncol,
                             const double *cols, char *out, int64_t cap);
/* Parses n such rows from text[0..len); returns the rows read. */
int64_t sph_parse_hexa_rows(const char *text, int64_t len, int64_t n, int32_t ncol, int64_t *id,
                            int64_t *istar, double *cols);
/* Snapshot rows (HelmholtzGas::writeAscii, hdr_hgas.hpp:136-180): kinds[k]
 * is 'e' (" %+e"), 'c' (" %+.3e") or 'd' (" %6lld" of the value). */
int64_t sph_format_ascii_rows(int64_t n, const int64_t *id, const int64_t *istar, int32_t ncol,
                              const double *cols, const char *kinds, char *out, int64_t cap);

/* ------------------------------------------------------------------------ */
/* ABI self-description, used by the tests to check the struct layouts.
 * Writes up to n int64 values: for each struct in the order DensityEPI,
 * DensityEPJ, Density, HydroEPI, HydroEPJ, Hydro, GravityEPI, GravityEPJ,
 * GravitySPJ, Gravity: sizeof followed by the byte offset of every field in
 * declaration order.  Returns the number of values available. */
int64_t sph_abi_layout(int64_t *out, int64_t n);

/* Library version string. */
const char *sph_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SPH_GB300_H */
