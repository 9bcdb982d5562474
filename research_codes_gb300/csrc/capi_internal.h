// capi_internal.h — context state behind the C ABI (not installed).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

#include "../../include/sph_gb300.h"
#include "pair_kernels.cuh"

#define PAIR_WARPS 4
// the FP64 hydro kernel's shared rings need half the warps per block to stay
// within the 48 KB static shared-memory limit
#define HYDRO64_WARPS 2

namespace sphrt {

// Device buffer that grows on demand (never inside stream capture).
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t cap = 0;
    int ensure(size_t n) {
        if (n <= cap && p) return 0;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = n + n / 4 + 64;
        if (cudaMalloc(&p, want * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return 1;
        }
        // no buffer is ever read before it is written, but a field that a
        // caller leaves unset (e.g. the signal velocity before the first
        // force evaluation) then holds zeros, not stale memory
        if (cudaMemset(p, 0, want * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(p);
            p = nullptr;
            return 1;
        }
        cap = want;
        return 0;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// Pinned host buffer that grows on demand.
template <class T>
struct HostBuf {
    T *p = nullptr;
    size_t cap = 0;
    int ensure(size_t n) {
        if (n <= cap && p) return 0;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        size_t want = n + n / 4 + 64;
        if (cudaMallocHost(&p, want * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return 1;
        }
        cap = want;
        return 0;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

// Buffers and dispatch state of one interaction kind (density/hydro/gravity).
struct KindState {
    HostBuf<char> h_in, h_out;
    DevBuf<char> d_in, d_out;
    DevBuf<dbl4> a4[8];
    DevBuf<float4> f4[16];   // FP32C double-float records
    DevBuf<int> hl_list, hl_cnt;       // FP32C hydro: marked-pair rows and counts
    DevBuf<int2> hl_ovf;               // FP32C hydro: overflowed rows (particle, walk)
    DevBuf<double2> a2[2];
    DevBuf<long long> id[2];
    DevBuf<double> d1[2];
    DevBuf<double> o[5];
    DevBuf<long long> o_np;
    DevBuf<unsigned char> o_itr;
    DevBuf<int> amb_i, amb_w;          // FP64 re-check queue of the density
    DevBuf<int4> fitems;
    std::vector<int4> items;
    std::vector<int> i_off;
    bool pending = false;
    int n_walk = 0;
    int flag_slot = 0;

    int ensure_density(size_t ni, size_t nj) {
        int e = 0;
        e |= a4[0].ensure(ni) | a4[1].ensure(ni) | id[0].ensure(ni) | d1[0].ensure(ni) | d1[1].ensure(ni);
        e |= a4[2].ensure(nj) | a4[3].ensure(nj) | id[1].ensure(nj);
        for (int k = 0; k < 5; ++k) e |= o[k].ensure(ni);
        e |= o_np.ensure(ni) | o_itr.ensure(ni);
        for (int k = 0; k < 4; ++k) e |= f4[k].ensure(ni) | f4[4 + k].ensure(nj);
        return e;
    }
    int ensure_hydro(size_t ni, size_t nj) {
        int e = 0;
        e |= a4[0].ensure(ni) | a4[1].ensure(ni) | a4[4].ensure(ni) | a4[5].ensure(ni);
        e |= a2[0].ensure(ni) | id[0].ensure(ni);
        e |= a4[2].ensure(nj) | a4[3].ensure(nj) | a4[6].ensure(nj) | a4[7].ensure(nj);
        e |= a2[1].ensure(nj) | id[1].ensure(nj);
        e |= o[0].ensure(3 * ni) | o[1].ensure(3 * ni);
        for (int k = 2; k < 5; ++k) e |= o[k].ensure(ni);
        for (int k = 0; k < 4; ++k) e |= f4[k].ensure(ni) | f4[4 + k].ensure(nj);
        for (int k = 8; k < 11; ++k) e |= f4[k].ensure(ni) | f4[k + 3].ensure(nj);
        e |= f4[14].ensure(ni) | f4[15].ensure(nj);
        e |= hl_list.ensure(ni * sphk::HYDRO_LIST_CAP) | hl_cnt.ensure(ni) | hl_ovf.ensure(ni);
        return e;
    }
    int ensure_gravity(size_t ni, size_t nj) {
        int e = 0;
        e |= a4[0].ensure(ni) | a4[2].ensure(nj) | d1[0].ensure(nj);
        e |= o[0].ensure(3 * ni) | o[1].ensure(ni) | o[2].ensure(ni);
        e |= f4[0].ensure(ni) | f4[1].ensure(ni) | f4[4].ensure(nj) | f4[5].ensure(nj);
        return e;
    }
    void release() {
        h_in.release();
        h_out.release();
        d_in.release();
        d_out.release();
        for (auto &b : a4) b.release();
        for (auto &b : f4) b.release();
        hl_list.release();
        hl_cnt.release();
        hl_ovf.release();
        for (auto &b : a2) b.release();
        for (auto &b : id) b.release();
        for (auto &b : d1) b.release();
        for (auto &b : o) b.release();
        o_np.release();
        o_itr.release();
        amb_i.release();
        amb_w.release();
        fitems.release();
    }
};

}  // namespace sphrt

struct sph_context {
    sph_params prm;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    int *d_queue = nullptr;   // [0..2] work-queue counters, [3] density re-check count,
                              // [4..6] finite flags, [7] re-check item count,
                              // [8] FP32C hydro rows that overflowed
    int *h_flags = nullptr;   // pinned copies of the flags
    int grid[3][2] = {{0}};   // persistent grid per kind and precision
    int grid_df = 0;          // resident blocks of the double-float hydro pass
    int grid_g64 = 0;         // persistent grid of the FP32C gravity kernel with a 64-entry j-tile
    sphrt::KindState kind[3];
    int n_systems = 0;        // live sph_system objects using this context
    char err[512] = {0};
};

namespace sphrt {
extern const float AMB_TOL;
int set_error(sph_context *ctx, int status, const char *fmt, ...);
int cuda_error(sph_context *ctx, cudaError_t e, const char *what);
int pair_grid(const sph_context *ctx, int kind, int precision, int n_items);
void launch_density(const sphk::DensityArgs &a, int precision, int grid, cudaStream_t s);
void launch_hydro(const sphk::HydroArgs &a, int precision, int grid, cudaStream_t s, int dfgrid,
                  cudaEvent_t mid = nullptr, bool mid_external = false);
void launch_gravity(const sphk::GravityArgs &a, int precision, int grid, cudaStream_t s, int jtile);
}  // namespace sphrt
