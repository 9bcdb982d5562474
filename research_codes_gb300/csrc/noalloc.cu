// noalloc.cu — sph_calc_gravity_ep_noalloc: the gravity functor for callers
// that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: host code that must not synchronise
// the device (an allocation can synchronise it), such as a hook another
// library calls on its hot path, embedded runtimes that own all device memory
// through a fixed arena, and loops that cannot afford an allocation's latency
// or its failure in mid-run.  (Not CUDA stream callbacks or cudaLaunchHostFunc
// functions: no CUDA call is allowed there, and this one launches kernels.)
// Such a caller still has its input and output buffers in device memory.  This entry point works on those buffers and keeps its own scratch
// (the FP32 double-float records, the per-particle results before they are
// added to the caller's forces, the work items and the work-queue counter) in
// one file-scope __device__ array, so it allocates nothing.
//
// The array is part of the library's device image: every GPU that loads the
// library holds it (about 2.4 MB) until the process exits.  Its size bounds a
// call to n_i <= SPH_NOALLOC_MAX_I and n_j <= SPH_NOALLOC_MAX_J.  Every call
// shares it and it keeps the last call's contents; the call clears the
// work-queue counter itself before the kernels use it.  Calls that overlap on
// the GPU (different streams, or different host threads on one device) race
// on the shared array and must be serialised by the caller.
//
// The array's device address is looked up on every call, with the caller's
// device current (cheap once the library's module is loaded on that device;
// nothing is cached, so a device reset leaves no stale pointer).  The first
// call on a device may load the module (CUDA loads modules lazily), which can
// allocate and synchronise: make that first call during set-up, before any
// stream capture.
#include <cuda_runtime.h>

#include "../../include/sph_gb300.h"
#include "pair_kernels.cuh"

namespace {

constexpr int MAX_I = SPH_NOALLOC_MAX_I;
constexpr int MAX_J = SPH_NOALLOC_MAX_J;
constexpr int NOALLOC_WARPS = 4;
constexpr int MAX_ITEMS = (MAX_I + 31) / 32;

// Layout of the scratch array (byte offsets, each 256-byte aligned).
constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t OFF_FI_HI = 0;
constexpr size_t OFF_FI_LO = align256(OFF_FI_HI + sizeof(float4) * MAX_I);
constexpr size_t OFF_FJ_HI = align256(OFF_FI_LO + sizeof(float4) * MAX_I);
constexpr size_t OFF_FJ_LO = align256(OFF_FJ_HI + sizeof(float4) * MAX_J);
constexpr size_t OFF_ACC = align256(OFF_FJ_LO + sizeof(float4) * MAX_J);
constexpr size_t OFF_POT = align256(OFF_ACC + sizeof(double) * 3 * MAX_I);
constexpr size_t OFF_ETA = align256(OFF_POT + sizeof(double) * MAX_I);
constexpr size_t OFF_ITEMS = align256(OFF_ETA + sizeof(double) * MAX_I);
constexpr size_t OFF_JOFF = align256(OFF_ITEMS + sizeof(sphk::WorkItem) * MAX_ITEMS);
constexpr size_t OFF_QUEUE = align256(OFF_JOFF + sizeof(int) * 2);
constexpr size_t SCRATCH_BYTES = align256(OFF_QUEUE + sizeof(int));

static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];


// Unpacks the caller's AoS inputs into double-float records, writes the work
// items (chunks of <= 32 i-particles) and the j range, clears the queue.
__global__ void noalloc_prepare(const sph_GravityEPI *epi, int ni, const sph_GravityEPJ *epj, int nj,
                                unsigned char *scr) {
    float4 *fi_hi = reinterpret_cast<float4 *>(scr + OFF_FI_HI);
    float4 *fi_lo = reinterpret_cast<float4 *>(scr + OFF_FI_LO);
    float4 *fj_hi = reinterpret_cast<float4 *>(scr + OFF_FJ_HI);
    float4 *fj_lo = reinterpret_cast<float4 *>(scr + OFF_FJ_LO);
    sphk::WorkItem *items = reinterpret_cast<sphk::WorkItem *>(scr + OFF_ITEMS);
    const int stride = gridDim.x * blockDim.x;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    for (int k = t; k < ni; k += stride) {
        const sph_GravityEPI e = epi[k];
        const float2 x = sphk::df_split(e.pos[0]), y = sphk::df_split(e.pos[1]), z = sphk::df_split(e.pos[2]);
        fi_hi[k] = make_float4(x.x, y.x, z.x, 0.0f);
        fi_lo[k] = make_float4(x.y, y.y, z.y, (float)e.eps2);
    }
    for (int k = t; k < nj; k += stride) {
        const sph_GravityEPJ e = epj[k];
        const float2 x = sphk::df_split(e.pos[0]), y = sphk::df_split(e.pos[1]), z = sphk::df_split(e.pos[2]);
        fj_hi[k] = make_float4(x.x, y.x, z.x, (float)e.mass);
        fj_lo[k] = make_float4(x.y, y.y, z.y, (float)e.eps2);
    }
    const int n_items = (ni + 31) / 32;
    for (int k = t; k < n_items; k += stride)
        items[k] = make_int4(0, 32 * k, min(32, ni - 32 * k), nj * min(32, ni - 32 * k));
    if (t == 0) {
        int *j_off = reinterpret_cast<int *>(scr + OFF_JOFF);
        j_off[0] = 0;
        j_off[1] = nj;
        *reinterpret_cast<int *>(scr + OFF_QUEUE) = 0;
    }
}

// force[k] += result[k] (calcGravity accumulates, hdr_gravity.hpp:333-337)
__global__ void noalloc_accumulate(int ni, const unsigned char *scr, sph_Gravity *force) {
    const double *acc = reinterpret_cast<const double *>(scr + OFF_ACC);
    const double *pot = reinterpret_cast<const double *>(scr + OFF_POT);
    const double *eta = reinterpret_cast<const double *>(scr + OFF_ETA);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ni; k += gridDim.x * blockDim.x) {
        sph_Gravity f = force[k];
        f.acc[0] += acc[3 * k];
        f.acc[1] += acc[3 * k + 1];
        f.acc[2] += acc[3 * k + 2];
        f.pot += pot[k];
        f.eta += eta[k];
        force[k] = f;
    }
}

// Device address of g_noalloc_scratch on the current device.
int scratch_address(unsigned char **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();   // this call's own lookup error
        return e == cudaErrorNoDevice || e == cudaErrorInvalidDevice ? SPH_ERR_NO_DEVICE : SPH_ERR_CUDA;
    }
    *out = static_cast<unsigned char *>(p);
    return SPH_OK;
}

}  // namespace

extern "C" int sph_calc_gravity_ep_noalloc(const sph_GravityEPI *epi, int32_t n_i, const sph_GravityEPJ *epj,
                                           int32_t n_j, sph_Gravity *force, void *stream) {
    if (n_i < 0 || n_j < 0 || (n_i > 0 && (!epi || !force)) || (n_j > 0 && !epj))
        return SPH_ERR_INVALID_ARGUMENT;
    if (n_i > MAX_I || n_j > MAX_J) return SPH_ERR_CAPACITY;
    if (n_i == 0) return SPH_OK;
    // an error left by the caller's earlier work is reported, not consumed
    if (cudaPeekAtLastError() != cudaSuccess) return SPH_ERR_CUDA;
    unsigned char *scr = nullptr;
    int st = scratch_address(&scr);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int pb = (n_j + n_i + 255) / 256;
    noalloc_prepare<<<pb < 1024 ? pb : 1024, 256, 0, s>>>(epi, n_i, epj, n_j, scr);
    if (cudaGetLastError() != cudaSuccess) return SPH_ERR_CUDA;   // this launch's own error
    sphk::GravityArgs a;
    a.i_pe = nullptr; a.j_pm = nullptr; a.j_eps2 = nullptr; a.s_pm = nullptr; a.s_eps2 = nullptr;
    a.s_quad = nullptr; a.f_sq0 = nullptr; a.f_sq1 = nullptr;
    a.fi_phi = reinterpret_cast<const float4 *>(scr + OFF_FI_HI);
    a.fi_plo = reinterpret_cast<const float4 *>(scr + OFF_FI_LO);
    a.f_phi = reinterpret_cast<const float4 *>(scr + OFF_FJ_HI);
    a.f_plo = reinterpret_cast<const float4 *>(scr + OFF_FJ_LO);
    a.f_shi = a.f_phi;
    a.f_slo = a.f_plo;
    a.n_split = 0x7fffffff;
    a.items = reinterpret_cast<const sphk::WorkItem *>(scr + OFF_ITEMS);
    a.n_items = (n_i + 31) / 32;
    a.n_items_dev = nullptr;
    a.j_off = reinterpret_cast<const int *>(scr + OFF_JOFF);
    a.j_idx = nullptr;
    a.i_list = nullptr;
    a.queue = reinterpret_cast<int *>(scr + OFF_QUEUE);
    a.o_acc = reinterpret_cast<double *>(scr + OFF_ACC);
    a.o_pot = reinterpret_cast<double *>(scr + OFF_POT);
    a.o_eta = reinterpret_cast<double *>(scr + OFF_ETA);
    const int blocks = (a.n_items + NOALLOC_WARPS - 1) / NOALLOC_WARPS;
    sphk::gravity_kernel<false, NOALLOC_WARPS><<<blocks, NOALLOC_WARPS * 32, 0, s>>>(a);
    if (cudaGetLastError() != cudaSuccess) return SPH_ERR_CUDA;
    noalloc_accumulate<<<(n_i + 255) / 256, 256, 0, s>>>(n_i, scr, force);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}
