// capi.cu — the C ABI of include/sph_gb300.h: contexts, the single-group
// functors and the batched Dispatch/Retrieve pairs.
//
// Data path of one dispatch (one CUDA stream per context):
//   host  : walk arrays -> one pinned staging buffer [offsets | items | EPI | EPJ]
//   H2D   : one cudaMemcpyAsync of that buffer
//   device: unpack kernel (reference AoS structs -> FP64 SoA), persistent pair
//           kernel, pack kernel (SoA -> reference Force structs, finite check)
//   D2H   : one cudaMemcpyAsync into pinned memory
//   Retrieve waits on the stream and scatters to the caller's per-walk arrays.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#include "../../include/sph_gb300.h"
#include "capi_internal.h"
#include "pair_kernels.cuh"

// ---- ABI layout checks: the reference classes' member order and padding ----
#define SPH_OFF(T, f, v) static_assert(offsetof(T, f) == (v), #T "::" #f " offset")
SPH_OFF(sph_DensityEPI, id, 0); SPH_OFF(sph_DensityEPI, mass, 8); SPH_OFF(sph_DensityEPI, pos, 16);
SPH_OFF(sph_DensityEPI, vel, 40); SPH_OFF(sph_DensityEPI, ksr, 64); SPH_OFF(sph_DensityEPI, rs, 72);
static_assert(sizeof(sph_DensityEPI) == 80, "DensityEPI size");
SPH_OFF(sph_DensityEPJ, mass, 8); SPH_OFF(sph_DensityEPJ, vel, 40);
static_assert(sizeof(sph_DensityEPJ) == 64, "DensityEPJ size");
SPH_OFF(sph_Density, ksr, 32); SPH_OFF(sph_Density, np, 40); SPH_OFF(sph_Density, itr, 48);
static_assert(sizeof(sph_Density) == 56, "Density size");
SPH_OFF(sph_HydroEPI, pos, 8); SPH_OFF(sph_HydroEPI, ksr, 56); SPH_OFF(sph_HydroEPI, eta, 136);
static_assert(sizeof(sph_HydroEPI) == 144, "HydroEPI size");
SPH_OFF(sph_HydroEPJ, mass, 8); SPH_OFF(sph_HydroEPJ, ksr, 64); SPH_OFF(sph_HydroEPJ, eta, 144);
static_assert(sizeof(sph_HydroEPJ) == 152, "HydroEPJ size");
SPH_OFF(sph_Hydro, accg, 24); SPH_OFF(sph_Hydro, diffu, 64);
static_assert(sizeof(sph_Hydro) == 72, "Hydro size");
static_assert(sizeof(sph_GravityEPI) == 32 && sizeof(sph_GravityEPJ) == 40 &&
              sizeof(sph_GravitySPJ) == 40 && sizeof(sph_Gravity) == 40, "gravity sizes");
SPH_OFF(sph_GravityEPJ, pos, 8); SPH_OFF(sph_GravityEPJ, eps2, 32); SPH_OFF(sph_Gravity, eta, 32);

using sphk::WorkItem;

namespace sphrt {

// Relative band |h - rs| <= AMB_TOL * rs in which an FP32C density result is
// recomputed in FP64 (FP32 h carries ~1e-7 relative error).
const float AMB_TOL = 4.0e-6f;

int set_error(sph_context *ctx, int status, const char *fmt, ...) {
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
        va_end(ap);
    }
    return status;
}

int cuda_error(sph_context *ctx, cudaError_t e, const char *what) {
    return set_error(ctx, SPH_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

template <class K>
static int occupancy_grid(K kernel, int threads, int sm_count, int *out) {
    int nb = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, 0);
    if (e != cudaSuccess) return (int)e;
    *out = std::max(1, nb) * sm_count;
    return 0;
}

int init_grids(sph_context *ctx) {
    const int th = PAIR_WARPS * 32;
    int e = 0;
    e |= occupancy_grid(sphk::density_kernel<false, PAIR_WARPS>, th, ctx->sm_count, &ctx->grid[0][0]);
    e |= occupancy_grid(sphk::density_kernel<true, PAIR_WARPS>, th, ctx->sm_count, &ctx->grid[0][1]);
    e |= occupancy_grid(sphk::hydro_kernel<false, PAIR_WARPS>, th, ctx->sm_count, &ctx->grid[1][0]);
    e |= occupancy_grid(sphk::hydro_kernel<true, HYDRO64_WARPS>, HYDRO64_WARPS * 32, ctx->sm_count,
                        &ctx->grid[1][1]);
    e |= occupancy_grid(sphk::gravity_kernel<false, PAIR_WARPS>, th, ctx->sm_count, &ctx->grid[2][0]);
    e |= occupancy_grid(sphk::gravity_kernel<true, PAIR_WARPS>, th, ctx->sm_count, &ctx->grid[2][1]);
    e |= occupancy_grid(sphk::hydro_df_lists, sphk::HYDRO_DF_THREADS, ctx->sm_count, &ctx->grid_df);
    e |= occupancy_grid(sphk::gravity_kernel<false, PAIR_WARPS, 64>, th, ctx->sm_count, &ctx->grid_g64);
    return e;
}

int pair_grid(const sph_context *ctx, int kind, int precision, int n_items) {
    const int full = ctx->grid[kind][precision == SPH_PREC_FP64 ? 1 : 0];
    const int warps = (kind == 1 && precision == SPH_PREC_FP64) ? HYDRO64_WARPS : PAIR_WARPS;
    const int need = (n_items + warps - 1) / warps;
    return std::max(1, std::min(full, need));
}

void launch_density(const sphk::DensityArgs &a, int precision, int grid, cudaStream_t s) {
    if (precision == SPH_PREC_FP64)
        sphk::density_kernel<true, PAIR_WARPS><<<grid, PAIR_WARPS * 32, 0, s>>>(a);
    else
        sphk::density_kernel<false, PAIR_WARPS><<<grid, PAIR_WARPS * 32, 0, s>>>(a);
}

// FP32C: the signal-velocity / marking kernel, then the double-float pass
// over the marked-pair rows and over the overflowed particles (a.df_novf
// must be zero at launch; dfgrid: resident blocks of the double-float pass).
// mid (optional) is recorded between the two (as an external record node
// when mid_external: inside a stream capture).
void launch_hydro(const sphk::HydroArgs &a, int precision, int grid, cudaStream_t s, int dfgrid,
                  cudaEvent_t mid, bool mid_external) {
    auto record_mid = [&]() {
        if (mid) cudaEventRecordWithFlags(mid, s, mid_external ? cudaEventRecordExternal : cudaEventRecordDefault);
    };
    if (precision == SPH_PREC_FP64) {
        sphk::hydro_kernel<true, HYDRO64_WARPS><<<grid, HYDRO64_WARPS * 32, 0, s>>>(a);
        record_mid();
        return;
    }
    sphk::hydro_kernel<false, PAIR_WARPS><<<grid, PAIR_WARPS * 32, 0, s>>>(a);
    record_mid();
    if (a.n_i <= 0) return;
    const int need = (a.n_i + sphk::HYDRO_DF_THREADS - 1) / sphk::HYDRO_DF_THREADS;
    sphk::hydro_df_lists<<<std::max(1, std::min(need, dfgrid)), sphk::HYDRO_DF_THREADS, 0, s>>>(a);
    // one block per overflowed particle, up to one per SM and round
    sphk::hydro_df_sweep<<<std::max(1, std::min(a.n_i, 2 * dfgrid / 5 + 1)), sphk::HYDRO_SWEEP_THREADS, 0, s>>>(a);
}

// jtile: entries a warp stages per pass in FP32C (32 or 64; FP64 uses 32).
void launch_gravity(const sphk::GravityArgs &a, int precision, int grid, cudaStream_t s, int jtile) {
    if (precision == SPH_PREC_FP64)
        sphk::gravity_kernel<true, PAIR_WARPS><<<grid, PAIR_WARPS * 32, 0, s>>>(a);
    else if (jtile == 64)
        sphk::gravity_kernel<false, PAIR_WARPS, 64><<<grid, PAIR_WARPS * 32, 0, s>>>(a);
    else
        sphk::gravity_kernel<false, PAIR_WARPS><<<grid, PAIR_WARPS * 32, 0, s>>>(a);
}

}  // namespace sphrt

using namespace sphrt;

// ---------------------------------------------------------------- kernels
namespace {

__device__ __forceinline__ bool finite3(double a, double b, double c) {
    return isfinite(a) && isfinite(b) && isfinite(c);
}

__global__ void unpack_density_i(const sph_DensityEPI *in, int n, dbl4 *pm, dbl4 *vel,
                                 long long *id, double *ksr, double *rs) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const sph_DensityEPI e = in[k];
        pm[k] = make_dbl4(e.pos[0], e.pos[1], e.pos[2], e.mass);
        vel[k] = make_dbl4(e.vel[0], e.vel[1], e.vel[2], 0.0);
        id[k] = e.id;
        ksr[k] = e.ksr;
        rs[k] = e.rs;
    }
}

__global__ void unpack_density_j(const sph_DensityEPJ *in, int n, dbl4 *pm, dbl4 *vel,
                                 long long *id) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const sph_DensityEPJ e = in[k];
        pm[k] = make_dbl4(e.pos[0], e.pos[1], e.pos[2], e.mass);
        vel[k] = make_dbl4(e.vel[0], e.vel[1], e.vel[2], 0.0);
        id[k] = e.id;
    }
}

template <class T>
__global__ void unpack_hydro(const T *in, int n, bool has_mass, dbl4 *pm, dbl4 *vel,
                             long long *id, dbl4 *h1, dbl4 *h2, double2 *h3) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const T &e = in[k];
        double m = 0.0;
        if (has_mass) m = reinterpret_cast<const sph_HydroEPJ *>(&e)->mass;
        pm[k] = make_dbl4(e.pos[0], e.pos[1], e.pos[2], m);
        vel[k] = make_dbl4(e.vel[0], e.vel[1], e.vel[2], 0.0);
        id[k] = e.id;
        h1[k] = make_dbl4(e.hinv, e.pres, e.presc, e.bswt);
        h2[k] = make_dbl4(e.dens, e.vsnd, e.alph, e.alphu);
        h3[k] = make_double2(e.thrm, e.eta);
    }
}

__global__ void unpack_gravity_i(const sph_GravityEPI *in, int n, dbl4 *pe) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const sph_GravityEPI e = in[k];
        pe[k] = make_dbl4(e.pos[0], e.pos[1], e.pos[2], e.eps2);
    }
}

// GravityEPJ and GravitySPJ share one layout (mass, pos[3], eps2).
__global__ void unpack_gravity_j(const sph_GravityEPJ *in, int n, dbl4 *pm, double *eps2) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const sph_GravityEPJ e = in[k];
        pm[k] = make_dbl4(e.pos[0], e.pos[1], e.pos[2], e.mass);
        eps2[k] = e.eps2;
    }
}

__global__ void pack_density(int n, const double *dens, const double *divv, const double *rotv,
                             const double *grdh, const double *ksr, const long long *np,
                             const unsigned char *itr, sph_Density *out, int *flag) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        sph_Density d;
        d.dens = dens[k];
        d.divv = divv[k];
        d.rotv = rotv[k];
        d.grdh = grdh[k];
        d.ksr = ksr[k];
        d.np = np[k];
        d.itr = itr[k] != 0;
        out[k] = d;
        if (!(finite3(d.dens, d.divv, d.rotv) && finite3(d.grdh, d.ksr, 0.0))) atomicOr(flag, 1);
    }
}

__global__ void pack_hydro(int n, const double *acch, const double *accg, const double *udot,
                           const double *vsmx, const double *diffu, sph_Hydro *out, int *flag) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        sph_Hydro h;
        for (int c = 0; c < 3; ++c) {
            h.acch[c] = acch[3 * k + c];
            h.accg[c] = accg[3 * k + c];
        }
        h.udot = udot[k];
        h.vsmx = vsmx[k];
        h.diffu = diffu[k];
        out[k] = h;
        if (!(finite3(h.acch[0], h.acch[1], h.acch[2]) && finite3(h.accg[0], h.accg[1], h.accg[2]) &&
              finite3(h.udot, h.vsmx, h.diffu)))
            atomicOr(flag, 1);
    }
}

__global__ void pack_gravity(int n, const double *acc, const double *pot, const double *eta,
                             sph_Gravity *out, int *flag) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        sph_Gravity g;
        for (int c = 0; c < 3; ++c) g.acc[c] = acc[3 * k + c];
        g.pot = pot[k];
        g.eta = eta[k];
        out[k] = g;
        if (!(finite3(g.acc[0], g.acc[1], g.acc[2]) && finite3(g.pot, g.eta, 0.0))) atomicOr(flag, 1);
    }
}

inline int eltwise_grid(long long n) {
    long long b = (n + 255) / 256;
    return (int)std::max(1LL, std::min(b, 4096LL));
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Splits every walk into work items of <= 32 i-particles; largest first.
void build_items(int n_walk, const int *i_off, const int *j_off, std::vector<WorkItem> &items) {
    items.clear();
    for (int w = 0; w < n_walk; ++w) {
        const int ni = i_off[w + 1] - i_off[w];
        const int nj = j_off[w + 1] - j_off[w];
        for (int k = 0; k < ni; k += 32) {
            const int c = std::min(32, ni - k);
            const long long cost = (long long)nj * c;
            items.push_back(make_int4(w, i_off[w] + k, c, (int)std::min<long long>(cost, 0x7fffffff)));
        }
    }
    std::stable_sort(items.begin(), items.end(),
                     [](const WorkItem &a, const WorkItem &b) { return a.w > b.w; });
}

}  // namespace

// ---------------------------------------------------------------- context
extern "C" void sph_params_default(sph_params *p) {
    if (!p) return;
    p->device = 0;
    p->precision = SPH_PREC_FP32C;
    p->eta = 1.6;
    p->ksr_max = 0.0;
    p->max_walks = 1000;
    p->max_i = 1000000;
    p->max_j = 10000000;
    p->check_finite = 1;
}

extern "C" const char *sph_status_string(int s) {
    switch (s) {
        case SPH_OK: return "ok";
        case SPH_ERR_INVALID_ARGUMENT: return "invalid argument";
        case SPH_ERR_CAPACITY: return "capacity exceeded";
        case SPH_ERR_CUDA: return "CUDA error";
        case SPH_ERR_NONFINITE: return "non-finite value in an output";
        case SPH_ERR_NOT_CONVERGED: return "search radius expansion did not converge";
        case SPH_ERR_STATE: return "call out of sequence";
        case SPH_ERR_NO_DEVICE: return "no usable CUDA device";
        default: return "unknown status";
    }
}

extern "C" const char *sph_version(void) { return "sph_gb300 0.1 (sm_103a)"; }

extern "C" int sph_context_create(const sph_params *p, sph_context **out) {
    if (!out) return SPH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    sph_params prm;
    if (p) prm = *p; else sph_params_default(&prm);
    if (prm.precision != SPH_PREC_FP32C && prm.precision != SPH_PREC_FP64) return SPH_ERR_INVALID_ARGUMENT;
    if (!(prm.eta > 0.0) || prm.max_walks <= 0 || prm.max_i <= 0 || prm.max_j <= 0 ||
        prm.max_i > 0x7fffffffLL || prm.max_j > 0x7fffffffLL)
        return SPH_ERR_INVALID_ARGUMENT;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return SPH_ERR_NO_DEVICE;
    }
    if (prm.device < 0 || prm.device >= ndev) return SPH_ERR_NO_DEVICE;
    sph_context *ctx = new (std::nothrow) sph_context();
    if (!ctx) return SPH_ERR_CAPACITY;
    ctx->prm = prm;
    cudaError_t e = cudaSetDevice(prm.device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, prm.device);
    int cc_major = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&cc_major, cudaDevAttrComputeCapabilityMajor, prm.device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_queue, 9 * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_flags, 8 * sizeof(int));
    if (e == cudaSuccess && init_grids(ctx) != 0) e = cudaErrorInvalidDeviceFunction;
    if (e != cudaSuccess) {
        cudaGetLastError();
        int st = (e == cudaErrorNoKernelImageForDevice || e == cudaErrorInvalidDeviceFunction)
                     ? SPH_ERR_NO_DEVICE : SPH_ERR_CUDA;
        sph_context_destroy(ctx);
        return st;
    }
    *out = ctx;
    return SPH_OK;
}

extern "C" int sph_context_destroy(sph_context *ctx) {
    if (!ctx) return SPH_ERR_INVALID_ARGUMENT;
    // systems hold the context's stream: they must go first
    if (ctx->n_systems > 0)
        return set_error(ctx, SPH_ERR_STATE, "%d system(s) still use this context", ctx->n_systems);
    cudaSetDevice(ctx->prm.device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (int k = 0; k < 3; ++k) ctx->kind[k].release();
    if (ctx->d_queue) cudaFree(ctx->d_queue);
    if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SPH_OK;
}

extern "C" int sph_context_set_eta(sph_context *ctx, double eta) {
    if (!ctx || !(eta > 0.0)) return SPH_ERR_INVALID_ARGUMENT;
    ctx->prm.eta = eta;
    return SPH_OK;
}

extern "C" int sph_context_set_ksr_max(sph_context *ctx, double v) {
    if (!ctx || std::isnan(v)) return SPH_ERR_INVALID_ARGUMENT;
    ctx->prm.ksr_max = v;
    return SPH_OK;
}

extern "C" int sph_context_set_precision(sph_context *ctx, int32_t precision) {
    if (!ctx || (precision != SPH_PREC_FP32C && precision != SPH_PREC_FP64)) return SPH_ERR_INVALID_ARGUMENT;
    ctx->prm.precision = precision;
    return SPH_OK;
}

extern "C" int sph_context_stream(const sph_context *ctx, void **stream) {
    if (!ctx || !stream) return SPH_ERR_INVALID_ARGUMENT;
    *stream = (void *)ctx->stream;
    return SPH_OK;
}

namespace {
// Eight independent FMA chains per thread keep the FP32 pipe full.
__global__ void fma_probe(float *out, int iters, float b, float c) {
    float a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    for (int k = 0; k < iters; ++k) {
        a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
        a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
    }
    const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 1234.5f) out[0] = s;   // keeps the chains live
}
}  // namespace

extern "C" int sph_probe_fp32_peak(sph_context *ctx, double *tflops) {
    if (!ctx || !tflops) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->prm.device);
    float *d = nullptr;
    cudaEvent_t e0, e1;
    if (cudaMalloc(&d, sizeof(float)) != cudaSuccess) return sphrt::set_error(ctx, SPH_ERR_CUDA, "probe alloc");
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = ctx->sm_count * 8, iters = 1 << 16;
    fma_probe<<<blocks, threads, 0, ctx->stream>>>(d, 256, 0.999f, 1e-3f);   // warm-up
    cudaEventRecord(e0, ctx->stream);
    fma_probe<<<blocks, threads, 0, ctx->stream>>>(d, iters, 0.999f, 1e-3f);
    cudaEventRecord(e1, ctx->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (e != cudaSuccess) return sphrt::cuda_error(ctx, e, "probe");
    *tflops = 2.0 * 8.0 * (double)iters * threads * blocks / (ms * 1e-3) / 1e12;
    return SPH_OK;
}

extern "C" int sph_context_last_error(const sph_context *ctx, char *buf, size_t n) {
    if (!ctx || !buf || n == 0) return SPH_ERR_INVALID_ARGUMENT;
    std::snprintf(buf, n, "%s", ctx->err);
    return SPH_OK;
}

// ---------------------------------------------------------------- dispatch
namespace {

enum { K_DENS = 0, K_HYDRO = 1, K_GRAV = 2 };

// Validates walk counts and fills the int32 offsets.  n_extra (gravity SPJ
// counts) may be null.
int walk_offsets(sph_context *ctx, int32_t n_walk, const int32_t *n_i, const int32_t *n_j,
                 const int32_t *n_extra, std::vector<int> &i_off, std::vector<int> &j_off) {
    if (n_walk < 0) return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "n_walk < 0");
    if (n_walk > ctx->prm.max_walks)
        return set_error(ctx, SPH_ERR_CAPACITY, "n_walk %d > max_walks %d", n_walk, ctx->prm.max_walks);
    if (n_walk > 0 && (!n_i || !n_j)) return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "null counts");
    i_off.assign(n_walk + 1, 0);
    j_off.assign(n_walk + 1, 0);
    long long ti = 0, tj = 0;
    for (int w = 0; w < n_walk; ++w) {
        const long long e = n_extra ? n_extra[w] : 0;
        if (n_i[w] < 0 || n_j[w] < 0 || e < 0)
            return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "negative count in walk %d", w);
        ti += n_i[w];
        tj += n_j[w] + e;
        if (ti > ctx->prm.max_i) return set_error(ctx, SPH_ERR_CAPACITY, "i total %lld > max_i", ti);
        if (tj > ctx->prm.max_j) return set_error(ctx, SPH_ERR_CAPACITY, "j total %lld > max_j", tj);
        i_off[w + 1] = (int)ti;
        j_off[w + 1] = (int)tj;
    }
    return SPH_OK;
}

// Lays out [i_off | j_off | items | EPI | EPJ] in the kind's pinned staging
// buffer; returns offsets of the struct regions.
struct Layout {
    size_t off_ioff, off_joff, off_items, off_epi, off_epj, total;
};

Layout make_layout(int n_walk, size_t n_items, size_t bytes_epi, size_t bytes_epj) {
    Layout L;
    size_t o = 0;
    L.off_ioff = o; o = align_up(o + sizeof(int) * (n_walk + 1), 256);
    L.off_joff = o; o = align_up(o + sizeof(int) * (n_walk + 1), 256);
    L.off_items = o; o = align_up(o + sizeof(WorkItem) * n_items, 256);
    L.off_epi = o; o = align_up(o + bytes_epi, 256);
    L.off_epj = o; o = align_up(o + bytes_epj, 256);
    L.total = o;
    return L;
}

int stage_common(sph_context *ctx, KindState &ks, const std::vector<int> &i_off,
                 const std::vector<int> &j_off, size_t epi_size, size_t epj_size, Layout &L) {
    const int n_walk = (int)i_off.size() - 1;
    build_items(n_walk, i_off.data(), j_off.data(), ks.items);
    L = make_layout(n_walk, ks.items.size(), epi_size * (size_t)i_off[n_walk],
                    epj_size * (size_t)j_off[n_walk]);
    if (ks.h_in.ensure(L.total) || ks.d_in.ensure(L.total))
        return set_error(ctx, SPH_ERR_CUDA, "staging allocation of %zu bytes failed", L.total);
    char *h = ks.h_in.p;
    std::memcpy(h + L.off_ioff, i_off.data(), sizeof(int) * (n_walk + 1));
    std::memcpy(h + L.off_joff, j_off.data(), sizeof(int) * (n_walk + 1));
    if (!ks.items.empty()) std::memcpy(h + L.off_items, ks.items.data(), sizeof(WorkItem) * ks.items.size());
    return SPH_OK;
}

int upload(sph_context *ctx, KindState &ks, const Layout &L) {
    cudaError_t e = cudaMemcpyAsync(ks.d_in.p, ks.h_in.p, L.total, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_error(ctx, e, "H2D");
    return SPH_OK;
}

int finish_dispatch(sph_context *ctx, KindState &ks, int n_walk, const std::vector<int> &i_off,
                    size_t out_size) {
    const int ni = i_off[n_walk];
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(ctx, e, "kernel launch");
    if (ni > 0) {
        e = cudaMemcpyAsync(ks.h_out.p, ks.d_out.p, out_size * ni, cudaMemcpyDeviceToHost, ctx->stream);
        if (e != cudaSuccess) return cuda_error(ctx, e, "D2H");
    }
    e = cudaMemcpyAsync(&ctx->h_flags[ks.flag_slot], ctx->d_queue + 4 + ks.flag_slot, sizeof(int),
                        cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return cuda_error(ctx, e, "D2H flag");
    ks.pending = true;
    ks.n_walk = n_walk;
    ks.i_off = i_off;
    return SPH_OK;
}

int begin_kind(sph_context *ctx, KindState &ks) {
    if (!ctx) return SPH_ERR_INVALID_ARGUMENT;
    if (ks.pending)
        return set_error(ctx, SPH_ERR_STATE, "a dispatch of this kind is outstanding; retrieve it first");
    cudaError_t e = cudaSetDevice(ctx->prm.device);
    if (e != cudaSuccess) return cuda_error(ctx, e, "cudaSetDevice");
    // The pinned staging buffer may still feed a copy of an earlier dispatch
    // that failed after its upload was queued; never overwrite it in flight.
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_error(ctx, e, "stream synchronize");
    return SPH_OK;
}

int reset_queue_and_flag(sph_context *ctx, KindState &ks) {
    cudaError_t e = cudaMemsetAsync(ctx->d_queue + ks.flag_slot, 0, sizeof(int), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_queue + 4 + ks.flag_slot, 0, sizeof(int), ctx->stream);
    if (e != cudaSuccess) return cuda_error(ctx, e, "memset");
    return SPH_OK;
}

template <class F>
int retrieve_common(sph_context *ctx, KindState &ks, int32_t n_walk, const int32_t *n_i, F **force,
                    size_t out_size) {
    if (!ctx) return SPH_ERR_INVALID_ARGUMENT;
    if (!ks.pending) return set_error(ctx, SPH_ERR_STATE, "retrieve without a dispatch");
    cudaError_t e = cudaSetDevice(ctx->prm.device);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    ks.pending = false;
    if (e != cudaSuccess) return cuda_error(ctx, e, "stream synchronize");
    if (n_walk != ks.n_walk)
        return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "n_walk %d differs from dispatch %d", n_walk, ks.n_walk);
    if (n_walk > 0 && (!n_i || !force)) return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "null arrays");
    for (int w = 0; w < n_walk; ++w) {
        const int ni = ks.i_off[w + 1] - ks.i_off[w];
        if (n_i[w] != ni)
            return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "walk %d: n_i %d differs from dispatch %d", w, n_i[w], ni);
        if (ni > 0 && !force[w]) return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "null force[%d]", w);
        if (ni > 0) std::memcpy(force[w], ks.h_out.p + out_size * ks.i_off[w], out_size * ni);
    }
    if (ctx->prm.check_finite && ctx->h_flags[ks.flag_slot])
        return set_error(ctx, SPH_ERR_NONFINITE, "non-finite value in the outputs");
    return SPH_OK;
}

}  // namespace

extern "C" int sph_dispatch_density(sph_context *ctx, int32_t tag, int32_t n_walk,
                                    const sph_DensityEPI **epi, const int32_t *n_epi,
                                    const sph_DensityEPJ **epj, const int32_t *n_epj) {
    (void)tag;
    KindState *ksp = ctx ? &ctx->kind[K_DENS] : nullptr;
    int st = begin_kind(ctx, *ksp);
    if (st) return st;
    KindState &ks = *ksp;
    ks.flag_slot = K_DENS;
    std::vector<int> i_off, j_off;
    if ((st = walk_offsets(ctx, n_walk, n_epi, n_epj, nullptr, i_off, j_off))) return st;
    if (n_walk > 0 && (!epi || !epj)) return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "null walk arrays");
    Layout L;
    if ((st = stage_common(ctx, ks, i_off, j_off, sizeof(sph_DensityEPI), sizeof(sph_DensityEPJ), L))) return st;
    for (int w = 0; w < n_walk; ++w) {
        if ((n_epi[w] && !epi[w]) || (n_epj[w] && !epj[w]))
            return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "null array in walk %d", w);
        if (n_epi[w]) std::memcpy(ks.h_in.p + L.off_epi + sizeof(sph_DensityEPI) * i_off[w], epi[w], sizeof(sph_DensityEPI) * n_epi[w]);
        if (n_epj[w]) std::memcpy(ks.h_in.p + L.off_epj + sizeof(sph_DensityEPJ) * j_off[w], epj[w], sizeof(sph_DensityEPJ) * n_epj[w]);
    }
    const int ni = i_off[n_walk], nj = j_off[n_walk];
    if (ks.ensure_density(ni, nj)) return set_error(ctx, SPH_ERR_CUDA, "device allocation failed");
    if (ks.h_out.ensure(sizeof(sph_Density) * (size_t)std::max(ni, 1)) ||
        ks.d_out.ensure(sizeof(sph_Density) * (size_t)std::max(ni, 1)))
        return set_error(ctx, SPH_ERR_CUDA, "output allocation failed");
    if ((st = upload(ctx, ks, L))) return st;
    if ((st = reset_queue_and_flag(ctx, ks))) return st;
    char *d = ks.d_in.p;
    if (ni > 0)
        unpack_density_i<<<eltwise_grid(ni), 256, 0, ctx->stream>>>(
            (const sph_DensityEPI *)(d + L.off_epi), ni, ks.a4[0].p, ks.a4[1].p, ks.id[0].p, ks.d1[0].p, ks.d1[1].p);
    if (nj > 0)
        unpack_density_j<<<eltwise_grid(nj), 256, 0, ctx->stream>>>(
            (const sph_DensityEPJ *)(d + L.off_epj), nj, ks.a4[2].p, ks.a4[3].p, ks.id[1].p);
    const bool f32 = ctx->prm.precision == SPH_PREC_FP32C;
    if (f32 && ni > 0)
        sphk::make_density_records<<<eltwise_grid(ni), 256, 0, ctx->stream>>>(ni, ks.a4[0].p, ks.a4[1].p, ks.f4[0].p,
                                                                             ks.f4[1].p, ks.f4[2].p, ks.f4[3].p);
    if (f32 && nj > 0)
        sphk::make_density_records<<<eltwise_grid(nj), 256, 0, ctx->stream>>>(nj, ks.a4[2].p, ks.a4[3].p, ks.f4[4].p,
                                                                             ks.f4[5].p, ks.f4[6].p, ks.f4[7].p);
    if (!ks.items.empty()) {
        sphk::DensityArgs a{};
        a.n_eval = nullptr;
        a.i_pm = ks.a4[0].p; a.i_vel = ks.a4[1].p; a.i_id = ks.id[0].p; a.i_ksr = ks.d1[0].p; a.i_rs = ks.d1[1].p;
        a.j_pm = ks.a4[2].p; a.j_vel = ks.a4[3].p; a.j_id = ks.id[1].p;
        a.fi = sphk::F32Part{ks.f4[0].p, ks.f4[1].p, ks.f4[2].p, ks.f4[3].p};
        a.fj = sphk::F32Part{ks.f4[4].p, ks.f4[5].p, ks.f4[6].p, ks.f4[7].p};
        a.i_list = nullptr;
        a.items = (const WorkItem *)(d + L.off_items);
        a.n_items = (int)ks.items.size();
        a.n_items_dev = nullptr;
        a.j_off = (const int *)(d + L.off_joff);
        a.j_idx = nullptr;
        a.queue = ctx->d_queue + K_DENS;
        a.o_dens = ks.o[0].p; a.o_divv = ks.o[1].p; a.o_rotv = ks.o[2].p; a.o_grdh = ks.o[3].p;
        a.o_ksr = ks.o[4].p; a.o_np = ks.o_np.p; a.o_itr = ks.o_itr.p;
        a.eta_ksrh = ctx->prm.eta * sphk::KSRH;
        a.ksr_max = ctx->prm.ksr_max > 0.0 ? ctx->prm.ksr_max : std::numeric_limits<double>::infinity();
        a.ksr_max_dev = nullptr;
        const int cap = std::max(256, ni / 16);
        if (ks.amb_i.ensure(cap) || ks.amb_w.ensure(cap) || ks.fitems.ensure(cap))
            return set_error(ctx, SPH_ERR_CUDA, "allocation failed");
        a.amb_count = f32 ? ctx->d_queue + 3 : nullptr;
        a.amb_i = ks.amb_i.p;
        a.amb_w = ks.amb_w.p;
        a.amb_cap = cap;
        a.amb_tol = AMB_TOL;
        if (f32) {
            cudaError_t e = cudaMemsetAsync(ctx->d_queue + 3, 0, sizeof(int), ctx->stream);
            if (e != cudaSuccess) return cuda_error(ctx, e, "memset");
        }
        launch_density(a, ctx->prm.precision, pair_grid(ctx, K_DENS, ctx->prm.precision, a.n_items), ctx->stream);
        if (f32) {
            // FP64 recomputation of the particles queued as decision-ambiguous
            sphk::make_fixup_items<<<1, 256, 0, ctx->stream>>>(ctx->d_queue + 3, ks.amb_w.p, cap, ks.fitems.p,
                                                                ctx->d_queue + 7);
            cudaError_t e = cudaMemsetAsync(ctx->d_queue + K_DENS, 0, sizeof(int), ctx->stream);
            if (e != cudaSuccess) return cuda_error(ctx, e, "memset");
            sphk::DensityArgs f = a;
            f.items = ks.fitems.p;
            f.n_items_dev = ctx->d_queue + 7;
            f.i_list = ks.amb_i.p;
            f.amb_count = nullptr;
            launch_density(f, SPH_PREC_FP64, pair_grid(ctx, K_DENS, SPH_PREC_FP64, cap), ctx->stream);
        }
    }
    if (ni > 0)
        pack_density<<<eltwise_grid(ni), 256, 0, ctx->stream>>>(
            ni, ks.o[0].p, ks.o[1].p, ks.o[2].p, ks.o[3].p, ks.o[4].p, ks.o_np.p, ks.o_itr.p,
            (sph_Density *)ks.d_out.p, ctx->d_queue + 4 + K_DENS);
    return finish_dispatch(ctx, ks, n_walk, i_off, sizeof(sph_Density));
}

extern "C" int sph_retrieve_density(sph_context *ctx, int32_t tag, int32_t n_walk, const int32_t *n_i,
                                    sph_Density **force) {
    (void)tag;
    if (!ctx) return SPH_ERR_INVALID_ARGUMENT;
    return retrieve_common(ctx, ctx->kind[K_DENS], n_walk, n_i, force, sizeof(sph_Density));
}

extern "C" int sph_dispatch_hydro(sph_context *ctx, int32_t tag, int32_t n_walk,
                                  const sph_HydroEPI **epi, const int32_t *n_epi,
                                  const sph_HydroEPJ **epj, const int32_t *n_epj) {
    (void)tag;
    KindState *ksp = ctx ? &ctx->kind[K_HYDRO] : nullptr;
    int st = begin_kind(ctx, *ksp);
    if (st) return st;
    KindState &ks = *ksp;
    ks.flag_slot = K_HYDRO;
    std::vector<int> i_off, j_off;
    if ((st = walk_offsets(ctx, n_walk, n_epi, n_epj, nullptr, i_off, j_off))) return st;
    if (n_walk > 0 && (!epi || !epj)) return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "null walk arrays");
    Layout L;
    if ((st = stage_common(ctx, ks, i_off, j_off, sizeof(sph_HydroEPI), sizeof(sph_HydroEPJ), L))) return st;
    for (int w = 0; w < n_walk; ++w) {
        if ((n_epi[w] && !epi[w]) || (n_epj[w] && !epj[w]))
            return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "null array in walk %d", w);
        if (n_epi[w]) std::memcpy(ks.h_in.p + L.off_epi + sizeof(sph_HydroEPI) * i_off[w], epi[w], sizeof(sph_HydroEPI) * n_epi[w]);
        if (n_epj[w]) std::memcpy(ks.h_in.p + L.off_epj + sizeof(sph_HydroEPJ) * j_off[w], epj[w], sizeof(sph_HydroEPJ) * n_epj[w]);
    }
    const int ni = i_off[n_walk], nj = j_off[n_walk];
    if (ks.ensure_hydro(ni, nj)) return set_error(ctx, SPH_ERR_CUDA, "device allocation failed");
    if (ks.h_out.ensure(sizeof(sph_Hydro) * (size_t)std::max(ni, 1)) ||
        ks.d_out.ensure(sizeof(sph_Hydro) * (size_t)std::max(ni, 1)))
        return set_error(ctx, SPH_ERR_CUDA, "output allocation failed");
    if ((st = upload(ctx, ks, L))) return st;
    if ((st = reset_queue_and_flag(ctx, ks))) return st;
    char *d = ks.d_in.p;
    if (ni > 0)
        unpack_hydro<sph_HydroEPI><<<eltwise_grid(ni), 256, 0, ctx->stream>>>(
            (const sph_HydroEPI *)(d + L.off_epi), ni, false, ks.a4[0].p, ks.a4[1].p, ks.id[0].p,
            ks.a4[4].p, ks.a4[5].p, ks.a2[0].p);
    if (nj > 0)
        unpack_hydro<sph_HydroEPJ><<<eltwise_grid(nj), 256, 0, ctx->stream>>>(
            (const sph_HydroEPJ *)(d + L.off_epj), nj, true, ks.a4[2].p, ks.a4[3].p, ks.id[1].p,
            ks.a4[6].p, ks.a4[7].p, ks.a2[1].p);
    const bool f32 = ctx->prm.precision == SPH_PREC_FP32C;
    if (f32 && ni > 0)
        sphk::make_hydro_records<<<eltwise_grid(ni), 256, 0, ctx->stream>>>(
            ni, ks.a4[0].p, ks.a4[1].p, ks.a4[4].p, ks.a4[5].p, ks.a2[0].p, ks.f4[0].p, ks.f4[1].p, ks.f4[2].p,
            ks.f4[3].p, ks.f4[8].p, ks.f4[9].p, ks.f4[10].p, ks.f4[14].p);
    if (f32 && nj > 0)
        sphk::make_hydro_records<<<eltwise_grid(nj), 256, 0, ctx->stream>>>(
            nj, ks.a4[2].p, ks.a4[3].p, ks.a4[6].p, ks.a4[7].p, ks.a2[1].p, ks.f4[4].p, ks.f4[5].p, ks.f4[6].p,
            ks.f4[7].p, ks.f4[11].p, ks.f4[12].p, ks.f4[13].p, ks.f4[15].p);
    if (!ks.items.empty()) {
        sphk::HydroArgs a{};
        a.n_eval_near = nullptr;
        a.n_eval_far = nullptr;
        a.i_pm = ks.a4[0].p; a.i_vel = ks.a4[1].p; a.i_id = ks.id[0].p;
        a.i_h1 = ks.a4[4].p; a.i_h2 = ks.a4[5].p; a.i_h3 = ks.a2[0].p;
        a.j_pm = ks.a4[2].p; a.j_vel = ks.a4[3].p; a.j_id = ks.id[1].p;
        a.j_h1 = ks.a4[6].p; a.j_h2 = ks.a4[7].p; a.j_h3 = ks.a2[1].p;
        a.fi = sphk::F32Part{ks.f4[0].p, ks.f4[1].p, ks.f4[2].p, ks.f4[3].p};
        a.fj = sphk::F32Part{ks.f4[4].p, ks.f4[5].p, ks.f4[6].p, ks.f4[7].p};
        a.fi_g1 = ks.f4[8].p; a.fi_g2 = ks.f4[9].p; a.fi_g3 = ks.f4[10].p;
        a.fj_g1 = ks.f4[11].p; a.fj_g2 = ks.f4[12].p; a.fj_g3 = ks.f4[13].p;
        a.i_list = nullptr;
        a.items = (const WorkItem *)(d + L.off_items);
        a.n_items = (int)ks.items.size();
        a.n_items_dev = nullptr;
        a.j_off = (const int *)(d + L.off_joff);
        a.j_idx = nullptr;
        a.queue = ctx->d_queue + K_HYDRO;
        a.o_acch = ks.o[0].p; a.o_accg = ks.o[1].p; a.o_udot = ks.o[2].p; a.o_vsmx = ks.o[3].p;
        a.o_diffu = ks.o[4].p;
        a.fi_g4 = ks.f4[14].p; a.fj_g4 = ks.f4[15].p;
        a.df_list = ks.hl_list.p; a.df_cap = sphk::HYDRO_LIST_CAP; a.df_cnt = ks.hl_cnt.p;
        a.df_ovf = ks.hl_ovf.p; a.df_novf = ctx->d_queue + 8; a.n_i = ni;
        if (f32) {
            // walks without items leave their rows empty; no overflow yet
            cudaError_t e = cudaMemsetAsync(ks.hl_cnt.p, 0, sizeof(int) * (size_t)ni, ctx->stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_queue + 8, 0, sizeof(int), ctx->stream);
            if (e != cudaSuccess) return cuda_error(ctx, e, "memset");
        }
        launch_hydro(a, ctx->prm.precision, pair_grid(ctx, K_HYDRO, ctx->prm.precision, a.n_items), ctx->stream,
                     ctx->grid_df);
    }
    if (ni > 0)
        pack_hydro<<<eltwise_grid(ni), 256, 0, ctx->stream>>>(
            ni, ks.o[0].p, ks.o[1].p, ks.o[2].p, ks.o[3].p, ks.o[4].p, (sph_Hydro *)ks.d_out.p,
            ctx->d_queue + 4 + K_HYDRO);
    return finish_dispatch(ctx, ks, n_walk, i_off, sizeof(sph_Hydro));
}

extern "C" int sph_retrieve_hydro(sph_context *ctx, int32_t tag, int32_t n_walk, const int32_t *n_i,
                                  sph_Hydro **force) {
    (void)tag;
    if (!ctx) return SPH_ERR_INVALID_ARGUMENT;
    return retrieve_common(ctx, ctx->kind[K_HYDRO], n_walk, n_i, force, sizeof(sph_Hydro));
}

extern "C" int sph_dispatch_gravity(sph_context *ctx, int32_t tag, int32_t n_walk,
                                    const sph_GravityEPI **epi, const int32_t *n_epi,
                                    const sph_GravityEPJ **epj, const int32_t *n_epj,
                                    const sph_GravitySPJ **spj, const int32_t *n_spj) {
    (void)tag;
    KindState *ksp = ctx ? &ctx->kind[K_GRAV] : nullptr;
    int st = begin_kind(ctx, *ksp);
    if (st) return st;
    KindState &ks = *ksp;
    ks.flag_slot = K_GRAV;
    std::vector<int> i_off, j_off;
    if ((st = walk_offsets(ctx, n_walk, n_epi, n_epj, n_spj, i_off, j_off))) return st;
    if (n_walk > 0 && (!epi || !epj)) return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "null walk arrays");
    if (n_spj && !spj) return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "null spj");
    Layout L;
    if ((st = stage_common(ctx, ks, i_off, j_off, sizeof(sph_GravityEPI), sizeof(sph_GravityEPJ), L))) return st;
    static_assert(sizeof(sph_GravitySPJ) == sizeof(sph_GravityEPJ), "SPJ appended to EPJ");
    for (int w = 0; w < n_walk; ++w) {
        const int ns = n_spj ? n_spj[w] : 0;
        if ((n_epi[w] && !epi[w]) || (n_epj[w] && !epj[w]) || (ns && !spj[w]))
            return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "null array in walk %d", w);
        char *jdst = ks.h_in.p + L.off_epj + sizeof(sph_GravityEPJ) * j_off[w];
        if (n_epi[w]) std::memcpy(ks.h_in.p + L.off_epi + sizeof(sph_GravityEPI) * i_off[w], epi[w], sizeof(sph_GravityEPI) * n_epi[w]);
        if (n_epj[w]) std::memcpy(jdst, epj[w], sizeof(sph_GravityEPJ) * n_epj[w]);
        if (ns) std::memcpy(jdst + sizeof(sph_GravityEPJ) * n_epj[w], spj[w], sizeof(sph_GravitySPJ) * ns);
    }
    const int ni = i_off[n_walk], nj = j_off[n_walk];
    if (ks.ensure_gravity(ni, nj)) return set_error(ctx, SPH_ERR_CUDA, "device allocation failed");
    if (ks.h_out.ensure(sizeof(sph_Gravity) * (size_t)std::max(ni, 1)) ||
        ks.d_out.ensure(sizeof(sph_Gravity) * (size_t)std::max(ni, 1)))
        return set_error(ctx, SPH_ERR_CUDA, "output allocation failed");
    if ((st = upload(ctx, ks, L))) return st;
    if ((st = reset_queue_and_flag(ctx, ks))) return st;
    char *d = ks.d_in.p;
    if (ni > 0)
        unpack_gravity_i<<<eltwise_grid(ni), 256, 0, ctx->stream>>>((const sph_GravityEPI *)(d + L.off_epi), ni, ks.a4[0].p);
    if (nj > 0)
        unpack_gravity_j<<<eltwise_grid(nj), 256, 0, ctx->stream>>>((const sph_GravityEPJ *)(d + L.off_epj), nj, ks.a4[2].p, ks.d1[0].p);
    const bool f32 = ctx->prm.precision == SPH_PREC_FP32C;
    if (f32 && ni > 0)
        sphk::make_gravity_records_pe<<<eltwise_grid(ni), 256, 0, ctx->stream>>>(ni, ks.a4[0].p, ks.f4[0].p, ks.f4[1].p);
    if (f32 && nj > 0)
        sphk::make_gravity_records<<<eltwise_grid(nj), 256, 0, ctx->stream>>>(nj, ks.a4[2].p, ks.d1[0].p, ks.f4[4].p,
                                                                             ks.f4[5].p);
    if (!ks.items.empty()) {
        sphk::GravityArgs a{};
        a.i_pe = ks.a4[0].p;
        a.j_pm = ks.a4[2].p; a.j_eps2 = ks.d1[0].p;
        a.s_pm = ks.a4[2].p; a.s_eps2 = ks.d1[0].p;
        a.fi_phi = ks.f4[0].p; a.fi_plo = ks.f4[1].p;
        a.f_phi = ks.f4[4].p; a.f_plo = ks.f4[5].p; a.f_shi = ks.f4[4].p; a.f_slo = ks.f4[5].p;
        a.i_list = nullptr;
        a.n_split = 0x7fffffff;
        a.items = (const WorkItem *)(d + L.off_items);
        a.n_items = (int)ks.items.size();
        a.n_items_dev = nullptr;
        a.j_off = (const int *)(d + L.off_joff);
        a.j_idx = nullptr;
        a.queue = ctx->d_queue + K_GRAV;
        a.o_acc = ks.o[0].p; a.o_pot = ks.o[1].p; a.o_eta = ks.o[2].p;
        a.s_quad = nullptr; a.f_sq0 = nullptr; a.f_sq1 = nullptr;   // SPJ are monopoles
        launch_gravity(a, ctx->prm.precision, pair_grid(ctx, K_GRAV, ctx->prm.precision, a.n_items), ctx->stream, 32);
    }
    if (ni > 0)
        pack_gravity<<<eltwise_grid(ni), 256, 0, ctx->stream>>>(ni, ks.o[0].p, ks.o[1].p, ks.o[2].p,
                                                               (sph_Gravity *)ks.d_out.p, ctx->d_queue + 4 + K_GRAV);
    return finish_dispatch(ctx, ks, n_walk, i_off, sizeof(sph_Gravity));
}

extern "C" int sph_retrieve_gravity(sph_context *ctx, int32_t tag, int32_t n_walk, const int32_t *n_i,
                                    sph_Gravity **force) {
    (void)tag;
    if (!ctx) return SPH_ERR_INVALID_ARGUMENT;
    return retrieve_common(ctx, ctx->kind[K_GRAV], n_walk, n_i, force, sizeof(sph_Gravity));
}

// ---------------------------------------------------------------- functors
extern "C" int sph_calc_density(sph_context *ctx, const sph_DensityEPI *epi, int32_t n_i,
                                const sph_DensityEPJ *epj, int32_t n_j, sph_Density *force) {
    if (!ctx) return SPH_ERR_INVALID_ARGUMENT;
    if (n_i < 0 || n_j < 0 || (n_i && (!epi || !force)) || (n_j && !epj))
        return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "bad functor arguments");
    int st = sph_dispatch_density(ctx, 0, 1, &epi, &n_i, &epj, &n_j);
    if (st) return st;
    return sph_retrieve_density(ctx, 0, 1, &n_i, &force);
}

extern "C" int sph_calc_hydro(sph_context *ctx, const sph_HydroEPI *epi, int32_t n_i,
                              const sph_HydroEPJ *epj, int32_t n_j, sph_Hydro *force) {
    if (!ctx) return SPH_ERR_INVALID_ARGUMENT;
    if (n_i < 0 || n_j < 0 || (n_i && (!epi || !force)) || (n_j && !epj))
        return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "bad functor arguments");
    int st = sph_dispatch_hydro(ctx, 0, 1, &epi, &n_i, &epj, &n_j);
    if (st) return st;
    return sph_retrieve_hydro(ctx, 0, 1, &n_i, &force);
}

namespace {
int gravity_accumulate(sph_context *ctx, const sph_GravityEPI *epi, int32_t n_i,
                       const sph_GravityEPJ *epj, int32_t n_ep, const sph_GravitySPJ *spj,
                       int32_t n_sp, sph_Gravity *force) {
    if (!ctx) return SPH_ERR_INVALID_ARGUMENT;
    if (n_i < 0 || n_ep < 0 || n_sp < 0 || (n_i && (!epi || !force)) || (n_ep && !epj) || (n_sp && !spj))
        return set_error(ctx, SPH_ERR_INVALID_ARGUMENT, "bad functor arguments");
    int st = sph_dispatch_gravity(ctx, 0, 1, &epi, &n_i, &epj, &n_ep, &spj, &n_sp);
    if (st) return st;
    std::vector<sph_Gravity> tmp((size_t)std::max(n_i, 1));
    sph_Gravity *tp = tmp.data();
    st = sph_retrieve_gravity(ctx, 0, 1, &n_i, &tp);
    if (st && st != SPH_ERR_NONFINITE) return st;
    for (int k = 0; k < n_i; ++k) {
        for (int c = 0; c < 3; ++c) force[k].acc[c] += tmp[k].acc[c];
        force[k].pot += tmp[k].pot;
        force[k].eta += tmp[k].eta;
    }
    return st;
}
}  // namespace

extern "C" int sph_calc_gravity_ep(sph_context *ctx, const sph_GravityEPI *epi, int32_t n_i,
                                   const sph_GravityEPJ *epj, int32_t n_j, sph_Gravity *force) {
    return gravity_accumulate(ctx, epi, n_i, epj, n_j, nullptr, 0, force);
}

extern "C" int sph_calc_gravity_sp(sph_context *ctx, const sph_GravityEPI *epi, int32_t n_i,
                                   const sph_GravitySPJ *spj, int32_t n_j, sph_Gravity *force) {
    return gravity_accumulate(ctx, epi, n_i, nullptr, 0, spj, n_j, force);
}

// ---------------------------------------------------------------- layout
extern "C" int64_t sph_abi_layout(int64_t *out, int64_t n) {
    std::vector<int64_t> v;
#define S(T) v.push_back(sizeof(T))
#define F(T, f) v.push_back(offsetof(T, f))
    S(sph_DensityEPI); F(sph_DensityEPI, id); F(sph_DensityEPI, mass); F(sph_DensityEPI, pos);
    F(sph_DensityEPI, vel); F(sph_DensityEPI, ksr); F(sph_DensityEPI, rs);
    S(sph_DensityEPJ); F(sph_DensityEPJ, id); F(sph_DensityEPJ, mass); F(sph_DensityEPJ, pos);
    F(sph_DensityEPJ, vel);
    S(sph_Density); F(sph_Density, dens); F(sph_Density, divv); F(sph_Density, rotv);
    F(sph_Density, grdh); F(sph_Density, ksr); F(sph_Density, np); F(sph_Density, itr);
#define HYDRO_TAIL(T) F(T, ksr); F(T, hinv); F(T, pres); F(T, presc); F(T, bswt); F(T, dens); \
    F(T, vsnd); F(T, alph); F(T, alphu); F(T, thrm); F(T, eta)
    S(sph_HydroEPI); F(sph_HydroEPI, id); F(sph_HydroEPI, pos); F(sph_HydroEPI, vel);
    HYDRO_TAIL(sph_HydroEPI);
    S(sph_HydroEPJ); F(sph_HydroEPJ, id); F(sph_HydroEPJ, mass); F(sph_HydroEPJ, pos);
    F(sph_HydroEPJ, vel); HYDRO_TAIL(sph_HydroEPJ);
    S(sph_Hydro); F(sph_Hydro, acch); F(sph_Hydro, accg); F(sph_Hydro, udot); F(sph_Hydro, vsmx);
    F(sph_Hydro, diffu);
    S(sph_GravityEPI); F(sph_GravityEPI, pos); F(sph_GravityEPI, eps2);
    S(sph_GravityEPJ); F(sph_GravityEPJ, mass); F(sph_GravityEPJ, pos); F(sph_GravityEPJ, eps2);
    S(sph_GravitySPJ); F(sph_GravitySPJ, mass); F(sph_GravitySPJ, pos); F(sph_GravitySPJ, eps2);
    S(sph_Gravity); F(sph_Gravity, acc); F(sph_Gravity, pot); F(sph_Gravity, eta);
#undef S
#undef F
#undef HYDRO_TAIL
    const int64_t m = (int64_t)v.size();
    if (out)
        for (int64_t k = 0; k < std::min(m, n); ++k) out[k] = v[k];
    return m;
}
