// system.cu — the device-resident particle system: the reference's step loop
// (calcTimestep -> predict -> calcSPHKernel -> correct) entirely on the GPU,
// with the tree / list builder of tree.cuh standing in for FDPS and the pair
// kernels of pair_kernels.cuh doing the interactions.  Every launch reads its
// counts from device memory, so a whole step can be captured as a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#include <cub/cub.cuh>

#include "../../include/sph_gb300.h"
#include "capi_internal.h"
#include "adjoint.cuh"
#include "pair_kernels.cuh"
#include "tree.cuh"

using sphk::WorkItem;
using sphrt::DevBuf;
using sphrt::HostBuf;

namespace {

constexpr double KSRH = sphk::KSRH;
constexpr double INV_KSRH2 = 1.0 / (KSRH * KSRH);   // eps^2 = h^2 / ksrh^2 without an FP64 divide
constexpr int ITEM_SPLIT_NJ = 4096;   // default list length above which a walk's items are halved (down to 4 i)
// density neighbour lists: entries per lane (a lane with more sweeps) and
// the default list radius over the first-pass h (later passes whose h grew
// beyond it sweep)
constexpr int NBR_CAP = 96;
constexpr float NBR_SLACK = 1.03f;
constexpr float MAX_NBR_SLACK = 2.0f;
constexpr int RED_BLOCKS = 296;   // 2 x 148..152 SMs; fixed for deterministic sums
constexpr int RED_THREADS = 256;
constexpr int MAX_RED = 8;

// int scalars
// Every list entry is written through a pool chunk and list offsets are
// 32-bit: a pool of at most this many chunks keeps every scan of entry counts
// below 2^31 (lists that would need more are a capacity error).
constexpr long long MAX_POOL_CHUNKS = 0x7fffffffLL / sphtree::LIST_CHUNK;
constexpr int NBKT = 32;   // cost classes of work items (log2 of the estimated cost)
enum { S_NGROUPS = 0, S_NACTIVE, S_NITEMS, S_QUEUE, S_ERROR, S_UNCONV, S_TOTAL, S_ITERS, S_AMB, S_NFIX, S_AMBTOT,
       S_NTASKS, S_NROOTS, S_POOL, S_POOLERR, S_TQUEUE, S_POOLMAX, S_HOVF, S_SMALL, S_BKT,
       S_NI = S_BKT + 2 * NBKT + 2 };
// double scalars
enum { D_TIME = 0, D_DT, D_KSRMAX, D_EPSU, D_DTC, D_XC, D_YC, D_ZC, D_MC, D_EKIN, D_ETHM, D_EPOT,
       D_R2, D_DN, D_NI };
// 64-bit counters
enum { L_PAIRS_D = 0, L_PAIRS_H, L_PAIRS_G, L_LIST_D, L_LIST_H, L_LIST_G, L_PAIRS_D1, L_LIST_R, L_EVAL_D1,
       L_EVAL_DG1, L_EVAL_HN, L_EVAL_HF, L_DLISTED, L_DSWEPT, L_HSKIP, L_HTILES, L_HMARK, L_HSLOTS, L_NI };
// error bits
enum { E_STACK = 1, E_LISTCAP = 2, E_NOTCONV = 4, E_DTMIN = 8, E_BOUNDS = 16 };
// phase events
enum { EV_TREE_B = 0, EV_TREE_E, EV_DENS_B, EV_DENSK_B, EV_DENSK_E, EV_DENS_E, EV_GLIST_B, EV_GLIST_E, EV_GK_B,
       EV_GK_E, EV_HLIST_B, EV_HK_B, EV_HK_E, EV_END, EV_HK_MID, EV_N };

inline int grid_for(long long n, int threads = 256) {
    long long b = (n + threads - 1) / threads;
    return (int)std::max(1LL, std::min(b, 8192LL));
}

#define GRID_STRIDE(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// ---------------------------------------------------------------- reductions
// Two-stage deterministic reduction: RED_BLOCKS partials in a fixed order,
// then one block adds them in index order.
template <class F>
__global__ void __launch_bounds__(RED_THREADS) reduce_stage1(int n, F f, double *partial) {
    __shared__ double sh[MAX_RED][RED_THREADS];
    double acc[MAX_RED];
    for (int k = 0; k < F::K; ++k) acc[k] = F::identity();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) f(p, acc);
    for (int k = 0; k < F::K; ++k) sh[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int k = 0; k < F::K; ++k) sh[k][threadIdx.x] = F::op(sh[k][threadIdx.x], sh[k][threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x < F::K) partial[blockIdx.x * MAX_RED + threadIdx.x] = sh[threadIdx.x][0];
}

// One warp per value: lane l combines partials l, l+32, ... in order, then a
// fixed shuffle tree combines the lanes (the same order on every run).
template <class Op>
__device__ __forceinline__ double warp_combine(const double *partial, int nb, int k, int lane) {
    double a = Op::identity();
    for (int b = lane; b < nb; b += 32) a = Op::op(a, partial[b * MAX_RED + k]);
    for (int o = 16; o > 0; o >>= 1) a = Op::op(a, __shfl_xor_sync(0xffffffffu, a, o));
    return a;
}

template <class F>
__global__ void reduce_stage2(const double *partial, int nb, double *out) {
    const int k = threadIdx.x >> 5;
    if (k >= F::K) return;
    const double a = warp_combine<F>(partial, nb, k, threadIdx.x & 31);
    if ((threadIdx.x & 31) == 0) out[k] = a;
}

struct SumOp {
    __device__ static double identity() { return 0.0; }
    __device__ static double op(double a, double b) { return a + b; }
};
struct MinOp {
    __device__ static double identity() { return 1.0e300; }
    __device__ static double op(double a, double b) { return fmin(a, b); }
};

// centre of mass of star 0 (hdr_util.hpp:8-34 with istar = 0)
struct Star0Com : SumOp {
    static constexpr int K = 4;
    const dbl4 *pos;
    const int *istar;
    __device__ void operator()(int p, double *a) const {
        if (istar[p] != 0) return;
        const dbl4 x = pos[p];
        a[0] += x.w * x.x;
        a[1] += x.w * x.y;
        a[2] += x.w * x.z;
        a[3] += x.w;
    }
};

// density-weighted r^2 about star 0's centre, over all particles (hdr_util.hpp:497-505)
struct KsrMaxSums : SumOp {
    static constexpr int K = 2;
    const dbl4 *pos;
    const double *dens;
    const double *xc;   // D_XC.. (already divided by mass)
    __device__ void operator()(int p, double *a) const {
        const dbl4 x = pos[p];
        const double dx = x.x - xc[0], dy = x.y - xc[1], dz = x.z - xc[2];
        a[0] += dens[p] * (dx * dx + dy * dy + dz * dz);
        a[1] += dens[p];
    }
};

// per-particle time step, hdr_hgas.hpp:477-488
// (f32: the candidate steps in FP32 arithmetic; GB300's FP64 divide and
// square root cost tens of FP64 instructions each)
struct TimestepMin : MinOp {
    static constexpr int K = 1;
    const double *ksr, *vsmx, *divv, *accg1, *accg2;
    double c_dt, dt_max;
    bool f32;
    __device__ void operator()(int p, double *a) const {
        const double gx = accg1[3 * p] + accg2[3 * p], gy = accg1[3 * p + 1] + accg2[3 * p + 1],
                     gz = accg1[3 * p + 2] + accg2[3 * p + 2];
        double dth, dtd, dtg;
        if (f32) {
            const float c = (float)c_dt, h = (float)ksr[p], dv = (float)divv[p];
            dth = (double)(c * h / ((float)vsmx[p] * (float)KSRH));
            dtd = (dv < 0.0f) ? (double)(-c / dv) : dt_max;
            dtg = (double)(c * sqrtf(h / sqrtf((float)(gx * gx + gy * gy + gz * gz))));
        } else {
            dth = c_dt * ksr[p] / (vsmx[p] * KSRH);
            dtd = (divv[p] < 0.0) ? (-c_dt / divv[p]) : dt_max;
            dtg = c_dt * sqrt(ksr[p] / sqrt(gx * gx + gy * gy + gz * gz));
        }
        const double d = fmin(fmin(dth, dt_max), fmin(dtg, dtd));
        a[0] = fmin(a[0], d);
    }
};

// energy parts, hdr_hgas.hpp:630-634
struct Energy : SumOp {
    static constexpr int K = 3;
    const dbl4 *pos, *vel;
    const double *uene, *pot;
    __device__ void operator()(int p, double *a) const {
        const double m = pos[p].w;
        const dbl4 v = vel[p];
        a[0] += 0.5 * m * (v.x * v.x + v.y * v.y + v.z * v.z);
        a[1] += m * uene[p];
        a[2] += 0.5 * m * pot[p];
    }
};

struct UeneMin : MinOp {
    static constexpr int K = 1;
    const double *uene;
    __device__ void operator()(int p, double *a) const { a[0] = fmin(a[0], uene[p]); }
};

// Analysis of the state (the reference's post-processing scripts, run here
// on the device): particle set = all particles (star < 0) or those of one
// star (istar == star).
// density-weighted centre and velocity, analysis/common.py:71-90
struct DensCentre : SumOp {
    static constexpr int K = 7;
    const dbl4 *pos, *vel;
    const double *dens;
    const int *istar;
    int star;
    __device__ void operator()(int p, double *a) const {
        if (star >= 0 && istar[p] != star) return;
        const dbl4 x = pos[p], v = vel[p];
        const double d = dens[p];
        a[0] += d * x.x;
        a[1] += d * x.y;
        a[2] += d * x.z;
        a[3] += d * v.x;
        a[4] += d * v.y;
        a[5] += d * v.z;
        a[6] += d;
    }
};

// bound / unbound mass: e = |v - v_ref|^2 / 2 + pot + u > 0 is unbound,
// analysis/unbound_mass/unbound_mass.py:10-27
struct BoundMass : SumOp {
    static constexpr int K = 2;
    const dbl4 *pos, *vel;
    const double *pot, *uene;
    const int *istar;
    int star;
    double vx, vy, vz;
    __device__ void operator()(int p, double *a) const {
        if (star >= 0 && istar[p] != star) return;
        const dbl4 v = vel[p];
        const double dx = v.x - vx, dy = v.y - vy, dz = v.z - vz;
        const double e = 0.5 * (dx * dx + dy * dy + dz * dz) + pot[p] + uene[p];
        a[e > 0.0 ? 1 : 0] += pos[p].w;
    }
};

// mass within a radius of a point, energy_check/energy_check.py:50-68
struct MassWithin : SumOp {
    static constexpr int K = 1;
    const dbl4 *pos;
    const int *istar;
    int star;
    double cx, cy, cz, r;
    __device__ void operator()(int p, double *a) const {
        if (star >= 0 && istar[p] != star) return;
        const dbl4 x = pos[p];
        const double dx = x.x - cx, dy = x.y - cy, dz = x.z - cz;
        if (sqrt(dx * dx + dy * dy + dz * dz) < r) a[0] += x.w;
    }
};

struct StarComs : SumOp {    // both stars' centres (calcSystemSize, hdr_util.hpp:95-113)
    static constexpr int K = 8;
    const dbl4 *pos;
    const int *istar;
    __device__ void operator()(int p, double *a) const {
        const dbl4 x = pos[p];
        const int o = istar[p] == 0 ? 0 : 4;
        if (istar[p] > 1) return;
        a[o + 0] += x.w * x.x;
        a[o + 1] += x.w * x.y;
        a[o + 2] += x.w * x.z;
        a[o + 3] += x.w;
    }
};

// ---------------------------------------------------------------- small kernels
// Run parameters the reference derives from the initial state
// (hdr_hgas.hpp:961-970, 1335): ksrmax = the distance between the two stars'
// centres of mass (c: their mass-weighted sums and masses; the largest double
// for a single star), epsu = 1e-4 of the smallest u (already in dsc).
__global__ void upload_scalars(const double *c, double *dsc) {
    double ksrmax = DBL_MAX;
    if (c[3] > 0.0 && c[7] > 0.0) {
        const double dx = c[0] / c[3] - c[4] / c[7], dy = c[1] / c[3] - c[5] / c[7], dz = c[2] / c[3] - c[6] / c[7];
        ksrmax = sqrt(dx * dx + dy * dy + dz * dz);
    }
    dsc[D_KSRMAX] = ksrmax;
    dsc[D_EPSU] *= 1e-4;
}
__global__ void bbox_stage1(const dbl4 *pos, int n, double *partial) {
    __shared__ double sh[6][RED_THREADS];
    double b[6] = {1e300, 1e300, 1e300, -1e300, -1e300, -1e300};
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const dbl4 x = pos[p];
        b[0] = fmin(b[0], x.x); b[1] = fmin(b[1], x.y); b[2] = fmin(b[2], x.z);
        b[3] = fmax(b[3], x.x); b[4] = fmax(b[4], x.y); b[5] = fmax(b[5], x.z);
    }
    for (int k = 0; k < 6; ++k) sh[k][threadIdx.x] = b[k];
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] = fmin(sh[k][threadIdx.x], sh[k][threadIdx.x + s]);
            for (int k = 3; k < 6; ++k) sh[k][threadIdx.x] = fmax(sh[k][threadIdx.x], sh[k][threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x < 6) partial[blockIdx.x * MAX_RED + threadIdx.x] = sh[threadIdx.x][0];
}

struct MaxOp {
    __device__ static double identity() { return -1.0e300; }
    __device__ static double op(double a, double b) { return fmax(a, b); }
};

__global__ void bbox_stage2(const double *partial, int nb, double *box) {
    const int k = threadIdx.x >> 5;
    if (k >= 6) return;
    const double a = (k < 3) ? warp_combine<MinOp>(partial, nb, k, threadIdx.x & 31)
                             : warp_combine<MaxOp>(partial, nb, k, threadIdx.x & 31);
    if ((threadIdx.x & 31) == 0) box[k] = a;
}

struct Persist {          // state carried across steps (permuted on each re-sort)
    dbl4 *pos, *vel, *vel2;
    long long *id;
    int *istar, *orig;
    double *uene, *uene2, *alph, *alph2, *alphu, *alphu2, *ksr;
};

__global__ void permute(int n, const int *idx, Persist src, Persist dst) {
    GRID_STRIDE(p, n) {
        const int q = idx[p];
        dst.pos[p] = src.pos[q];
        dst.vel[p] = src.vel[q];
        dst.vel2[p] = src.vel2[q];
        dst.id[p] = src.id[q];
        dst.istar[p] = src.istar[q];
        dst.orig[p] = src.orig[q];
        dst.uene[p] = src.uene[q];
        dst.uene2[p] = src.uene2[q];
        dst.alph[p] = src.alph[q];
        dst.alph2[p] = src.alph2[q];
        dst.alphu[p] = src.alphu[q];
        dst.alphu2[p] = src.alphu2[q];
        dst.ksr[p] = src.ksr[q];
    }
}

// Softening of the first guess of h, for the refit after the tree build only
// (the refit after the density phase and the gravity kernel use post_density's).
__global__ void eps2_from_h(int n, const double *h, double *eps2) {
    GRID_STRIDE(p, n) { eps2[p] = h[p] * h[p] * INV_KSRH2; }
}

// compact group roots: position-indexed flags -> group arrays
__global__ void compact_groups(int n, const int *flag, const int *scan, const int *root_at,
                               sphtree::Nodes t, int *group_node, int *group_first, int *group_count,
                               int *scal) {
    GRID_STRIDE(p, n) {
        if (flag[p]) {
            const int g = scan[p];
            const int v = root_at[p];
            group_node[g] = v;
            group_first[g] = p;
            group_count[g] = t.count[v];
        }
        if (p == n - 1) scal[S_NGROUPS] = scan[p] + flag[p];
    }
}

// one warp per group: max rs over the members that are still iterating
__global__ void group_rs_max(const int *scal, const int *group_first, const int *group_count,
                             const double *rs, double *rmax, int *active_flag) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    const int ng = scal[S_NGROUPS];
    for (int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < ng; g += warps) {
        double m = 0.0;
        for (int k = lane; k < group_count[g]; k += 32) m = fmax(m, rs[group_first[g] + k]);
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) {
            rmax[g] = m;
            active_flag[g] = m > 0.0 ? 1 : 0;
        }
    }
}

__global__ void compact_active(int n, const int *scal, const int *flag, const int *scan,
                               const int *group_node, const int *group_first, const int *group_count,
                               const double *rmax, int *a_node, int *a_first, int *a_count, double *a_r,
                               int *scal_out) {
    const int ng = scal[S_NGROUPS];
    GRID_STRIDE(g, n) {
        if (g < ng && flag[g]) {
            const int k = scan[g];
            a_node[k] = group_node[g];
            a_first[k] = group_first[g];
            a_count[k] = group_count[g];
            a_r[k] = rmax[g];
        }
        if (g == n - 1) scal_out[S_NACTIVE] = scan[g] + flag[g];
    }
}

__global__ void set_int(int *p, int v) { *p = v; }
__global__ void accumulate_int(const int *src, int *dst) { *dst += *src; }
__global__ void copy_int(const int *src, int *dst) { *dst = *src; }

// list totals: offset[n-1] + count[n-1] (counts beyond the walk count are 0)
// Task count of a list build (clamped to the task capacity, error bit beyond).
__global__ void task_total(int n, const int *toff, int cap, int *scal) {
    const int t = toff[n];
    scal[S_NTASKS] = t < cap ? t : cap;
    if (t > cap) atomicOr(&scal[S_ERROR], E_LISTCAP);
}

__global__ void list_total(int n, const int *cnt, const int *off, long long cap, int *scal, long long *lscal,
                           int lslot) {
    const long long tot = (long long)off[n - 1] + cnt[n - 1];
    scal[S_TOTAL] = (int)min(tot, (long long)0x7fffffff);
    lscal[lslot] = tot;
    if (tot > cap) atomicOr(&scal[S_ERROR], E_LISTCAP);
}

// work items: walk k gets ceil(n_i/chunk) items over its i-segment
// [i_first[k], i_first[k] + i_count[k]) (particle indices or positions in
// an index list)
// Item size of a walk: walks with long lists are cut into items of fewer
// i-particles (several lanes per i-particle, each lane a share of the list),
// so that no single item runs much longer than a warp's share of the phase.
__device__ __forceinline__ int item_chunk(int nj, int chunk, int split_nj) {
    int c = chunk;
    long long lim = split_nj;
    while (c > 4 && nj > lim) {
        c >>= 1;
        lim <<= 1;
    }
    return c;
}

// Cost class of an item of sz i-particles against nj j-entries: staging
// grows with nj, the pair loops with nj * sz.
__device__ __forceinline__ int cost_bucket(int nj, int sz) {
    const long long c = (long long)nj * (sz + 2) + 1;
    return min(NBKT - 1, 63 - __clzll(c));
}

// Histogram of the items of all walks over the cost classes (bkt[0..NBKT),
// zero on entry).
__global__ void item_buckets(int n, const int *n_walks, const int *i_count, const int *j_cnt, int chunk,
                             int split_nj, int *bkt) {
    const int nw = *n_walks;
    GRID_STRIDE(k, n) {
        if (k < nw) {
            const int ni = i_count[k], nj = j_cnt[k];
            const int ch = item_chunk(nj, chunk, split_nj);
            const int full = ni / ch, rest = ni - full * ch;
            if (full) atomicAdd(&bkt[cost_bucket(nj, ch)], full);
            if (rest) atomicAdd(&bkt[cost_bucket(nj, rest)], 1);
        }
    }
}

// Item order.  The items of the SPH_HEAVY_CLASSES most expensive nonempty
// cost classes go first, most expensive class first, so that the persistent
// kernels start the longest items early; all other items follow in walk
// order, so that warps running at the same time work on neighbouring walks
// and share their j records in L2.  Gravity lists are of nearly uniform
// length, so their items all stay in walk order (heavy = 0).  The order of
// items does not affect any result (every item owns its outputs).
#ifndef SPH_HEAVY_CLASSES
#define SPH_HEAVY_CLASSES 2
#endif

// bkt[0..NBKT): class counts (in); bkt[NBKT + b]: cursor of heavy class b;
// bkt[2 NBKT]: lowest heavy class; bkt[2 NBKT + 1]: number of heavy items.
__global__ void bucket_offsets(int *bkt, int heavy) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int bmax = -1;
        for (int b = NBKT - 1; b >= 0 && bmax < 0; --b)
            if (bkt[b] > 0) bmax = b;
        const int bh = bmax - heavy + 1;
        int acc = 0;
        for (int b = NBKT - 1; b >= 0; --b) {
            bkt[NBKT + b] = acc;
            if (b >= bh) acc += bkt[b];
        }
        bkt[2 * NBKT] = bh;
        bkt[2 * NBKT + 1] = acc;
    }
}

// Number of light items (class below the heavy ones) of each walk.
__global__ void light_counts(int n, const int *n_walks, const int *i_count, const int *j_cnt, int chunk,
                             int split_nj, const int *bkt, int *lc) {
    const int nw = *n_walks;
    const int bh = bkt[2 * NBKT];
    GRID_STRIDE(k, n + 1) {
        int c = 0;
        if (k < nw) {
            const int ni = i_count[k], nj = j_cnt[k];
            const int ch = item_chunk(nj, chunk, split_nj);
            for (int c0 = 0; c0 < ni; c0 += ch) c += cost_bucket(nj, min(ch, ni - c0)) < bh ? 1 : 0;
        }
        lc[k] = c;
    }
}

// A list build that overflowed its buffers (capacity or stack error set)
// leaves offsets that run past the list arrays: no pair kernel may read
// them, so the evaluation gets no work items (it is repeated, or reported).
__global__ void drop_items_on_overflow(int *scal) {
    if (scal[S_ERROR] & (E_LISTCAP | E_STACK)) scal[S_NITEMS] = 0;
}

__global__ void fill_items(int n, const int *n_walks, const int *i_first, const int *i_count, int chunk,
                           int split_nj, const int *j_cnt, int *bkt, const int *light_off, WorkItem *items,
                           int *n_items, long long *pairs) {
    const int nw = *n_walks;
    const int bh = bkt[2 * NBKT];
    const int n_heavy = bkt[2 * NBKT + 1];
    long long local = 0;
    GRID_STRIDE(k, n) {
        if (k < nw) {
            const int ni = i_count[k];
            const int nj = j_cnt[k];
            const int ch = item_chunk(nj, chunk, split_nj);
            int lpos = n_heavy + light_off[k];
            for (int c0 = 0; c0 < ni; c0 += ch) {
                const int sz = min(ch, ni - c0);
                const int b = cost_bucket(nj, sz);
                const int pos = (b >= bh) ? atomicAdd(&bkt[NBKT + b], 1) : lpos++;
                items[pos] = make_int4(k, i_first[k] + c0, sz, nj * sz);
            }
            local += (long long)ni * nj;
        }
        if (k == 0) *n_items = n_heavy + light_off[nw];
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd((unsigned long long *)pairs, (unsigned long long)local);
}

// particles still iterating (rs != 0) -> flags for the index list
__global__ void iterating_flags(int n, const double *rs, int *flag) {
    GRID_STRIDE(p, n) { flag[p] = rs[p] != 0.0 ? 1 : 0; }
}

__global__ void scatter_list(int n, const int *flag, const int *scan, int *list) {
    GRID_STRIDE(p, n) {
        if (flag[p]) list[scan[p]] = p;
    }
}

// Re-walks with at most REWALK_SMALL iterating particles run on
// density_rewalk_blocks (a block per walk) instead of density_kernel.
constexpr int REWALK_SMALL = 1024;
__global__ void rewalk_small(int n, const int *flag, const int *scan, int *scal) {
    const int total = scan[n - 1] + flag[n - 1];
    scal[S_SMALL] = (total <= REWALK_SMALL) ? 1 : 0;
}
__global__ void drop_items_if_small(int *scal) {
    if (scal[S_SMALL]) scal[S_NITEMS] = 0;
}

// the index-list segment of each active walk
__global__ void walk_segments(int n, const int *scal, const int *a_first, const int *a_count, const int *flag,
                              const int *scan, int *seg_first, int *seg_count) {
    const int nw = scal[S_NACTIVE];
    GRID_STRIDE(k, n) {
        if (k < nw) {
            const int f = a_first[k], e = a_first[k] + a_count[k];
            const int sf = scan[f];
            const int se = (e < n) ? scan[e] : scan[n - 1] + flag[n - 1];
            seg_first[k] = sf;
            seg_count[k] = se - sf;
        }
    }
}

__global__ void init_rs(int n, const double *ksr, double *rs) {
    GRID_STRIDE(p, n) { rs[p] = 1.1 * ksr[p]; }   // hdr_density.hpp:376-379
}

struct DensOut {
    double *dens, *divv, *rotv, *grdh, *ksr;
    long long *np;
    unsigned char *itr;
};

// hdr_density.hpp:401-411: converged particles take the result and get rs = 0,
// the others expand rs by 1.1 and stay in the iteration.
__global__ void commit_density(int n, double *rs, DensOut tmp, DensOut st, int *scal) {
    // after a list overflow no density item ran: the state stays as it was
    // for the repeated evaluation
    if (scal[S_ERROR] & (E_LISTCAP | E_STACK)) return;
    int local = 0;
    GRID_STRIDE(p, n) {
        if (rs[p] != 0.0) {
            if (tmp.itr[p]) {
                rs[p] *= 1.1;
                local = 1;
            } else {
                rs[p] = 0.0;
                st.dens[p] = tmp.dens[p];
                st.divv[p] = tmp.divv[p];
                st.rotv[p] = tmp.rotv[p];
                st.grdh[p] = tmp.grdh[p];
                st.ksr[p] = tmp.ksr[p];
                st.np[p] = tmp.np[p];
            }
        }
    }
    if (__any_sync(0xffffffffu, local) && (threadIdx.x & 31) == 0) atomicAdd(&scal[S_UNCONV], 1);
}

// end of a walk of the captured re-walk loop (its index on the device) and
// the loop's condition: another walk while particles iterate and walks remain
__global__ void iteration_end_loop(int *scal, int max_it, cudaGraphConditionalHandle h) {
    const int it = scal[S_ITERS] - 1;
    unsigned more = 0;
    if (scal[S_UNCONV] > 0) {
        scal[S_ITERS] = it + 2;
        if (it + 1 >= max_it) atomicOr(&scal[S_ERROR], E_NOTCONV);
        else more = 1;
    }
    scal[S_UNCONV] = 0;
    cudaGraphSetConditional(h, more);
}

// entry condition of the re-walk loop: the first walk left particles iterating
__global__ void rewalk_start(const int *scal, int max_it, cudaGraphConditionalHandle h) {
    cudaGraphSetConditional(h, (scal[S_ITERS] > 1 && max_it > 1) ? 1u : 0u);
}

__global__ void iteration_end(int *scal, int max_it, int it) {
    if (scal[S_UNCONV] > 0) {
        scal[S_ITERS] = it + 2;
        if (it + 1 >= max_it) atomicOr(&scal[S_ERROR], E_NOTCONV);
    }
    scal[S_UNCONV] = 0;
}

// EOS (hdr_hgas.hpp:339-342), Balsara (hdr_sph.hpp:79-81), softening eps^2.
// f32 (FP32C runs): sound speed and Balsara switch in FP32 arithmetic (they
// feed the FP32 pair records; FP64 divide and square root cost tens of FP64
// instructions each on GB300), with c = sqrt((1 + 1/n) P / rho) as
// sqrt((1 + 1/n) u / n); the FP64 engine keeps the reference's FP64 forms.
__global__ void post_density(int n, const dbl4 *pos, const double *dens, const double *uene,
                             const double *divv, const double *rotv, const double *ksr, double *pres,
                             double *vsnd, double *bswt, double *eps2, dbl4 *pe, bool f32) {
    const double ninv = 1.0 / 1.5;
    GRID_STRIDE(p, n) {
        const double P = ninv * dens[p] * uene[p];
        double c, b;
        if (f32) {
            const float cf = sqrtf((float)((1.0 + ninv) * ninv * uene[p]));
            const float ad = fabsf((float)divv[p]);
            c = (double)cf;
            b = (double)(ad / (ad + fabsf((float)rotv[p]) + 1e-4f * cf * (float)KSRH / (float)ksr[p]));
        } else {
            c = sqrt((1.0 + ninv) * P / dens[p]);
            const double ad = fabs(divv[p]);
            b = ad / (ad + fabs(rotv[p]) + 1e-4 * c * KSRH / ksr[p]);
        }
        pres[p] = P;
        vsnd[p] = c;
        bswt[p] = b;
        const double e2 = f32 ? ksr[p] * ksr[p] * INV_KSRH2 : (ksr[p] / KSRH) * (ksr[p] / KSRH);
        eps2[p] = e2;
        const dbl4 x = pos[p];
        pe[p] = make_dbl4(x.x, x.y, x.z, e2);
    }
}

// Gravity write-back, hdr_gravity.hpp:107-113
__global__ void gravity_writeback(int n, double G, const double *acc, const double *pot, const double *etas,
                                  const double *ksr, const double *grdh, const double *dens, double *accg2,
                                  double *pot_out, double *eta_out, bool f32) {
    GRID_STRIDE(p, n) {
        for (int c = 0; c < 3; ++c) accg2[3 * p + c] = G * acc[3 * p + c];
        if (f32) {   // eta feeds the FP32 hydro records
            const float h = (float)ksr[p];
            eta_out[p] = (double)(h * h / (float)(KSRH * KSRH) * (float)grdh[p] / (3.0f * (float)dens[p]) *
                                  (float)etas[p]);
        } else {
            eta_out[p] = ksr[p] * ksr[p] / (KSRH * KSRH) * grdh[p] / (3.0 * dens[p]) * etas[p];
        }
        pot_out[p] = G * pot[p];
    }
}

// Largest sound speed over each hydro walk's j-list (one block per walk, -inf
// for an empty list).  The signal velocity of every i-particle of the walk,
// a maximum of cs_i + cs_j - 3 min(w, 0) over the list (hdr_hydro.hpp:368-372),
// is at least its own sound speed plus this.
constexpr int CSMAX_THREADS = 256;
__global__ void __launch_bounds__(CSMAX_THREADS) walk_csmax(const int *n_walks, const int *j_off, const int *j_idx,
                                                            const float4 *f_g2, const dbl4 *h2, double *out,
                                                            const int *scal) {
    __shared__ double red[CSMAX_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (scal[S_ERROR] & (E_LISTCAP | E_STACK)) return;   // the lists overflowed (no hydro items either)
    const int nw = *n_walks;
    for (int w = blockIdx.x; w < nw; w += gridDim.x) {
        double m = -INFINITY;
        const int e = j_off[w + 1];
        // four entries per thread and round: their loads are in flight together
        for (int k = j_off[w] + threadIdx.x; k < e; k += 4 * CSMAX_THREADS) {
            int j[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int kk = k + u * CSMAX_THREADS;
                j[u] = kk < e ? (j_idx ? j_idx[kk] : kk) : -1;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (j[u] >= 0) m = fmax(m, f_g2 ? (double)f_g2[j[u]].y : h2[j[u]].y);   // NaN never raises it
        }
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) red[warp] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int k = 1; k < CSMAX_THREADS / 32; ++k) m = fmax(m, red[k]);
            out[w] = m;
        }
        __syncthreads();
    }
}

// HydroEPI/EPJ::copyFromFP, hdr_hydro.hpp:45-62 / 95-113 (umin = 0)
__global__ void hydro_prep(int n, const double *ksr, const double *pres, const double *grdh,
                           const double *dens, const double *bswt, const double *vsnd, const double *alph,
                           const double *alphu, const double *uene, const double *eta, dbl4 *h1, dbl4 *h2,
                           double2 *h3, bool f32) {
    (void)f32;
    GRID_STRIDE(p, n) {
        // FP64 in both precisions: the FP32C records carry 1/h, h^-4 and
        // P Omega / rho^2 as double-float splits for the cancelling sums
        const double hinv = 1.0 / ksr[p];
        const double presc = pres[p] * grdh[p] / (dens[p] * dens[p]);
        h1[p] = make_dbl4(hinv, pres[p], presc, 0.5 * bswt[p]);
        h2[p] = make_dbl4(dens[p], vsnd[p], alph[p], alphu[p]);
        h3[p] = make_double2(fmax(uene[p] - 0.0, 0.0), eta[p]);
    }
}

struct AlphaParams {
    double amax, amin, aumax, aumin;
};

// Hydro write-back (hdr_hydro.hpp:19-26), sumAcceleration (hdr_sph.hpp:95-97),
// calcAlphaDot (hdr_hgas.hpp:750-762)
__global__ void hydro_writeback(int n, double G, const double *acch_r, const double *accg_r,
                                const double *udot_r, const double *vsmx_r, const double *diffu_r,
                                double *acch, double *accg1, const double *accg2, double *acc, double *udot,
                                double *vsmx, double *diffu, const double *divv, const double *alph,
                                const double *alphu, const double *vsnd, const double *ksr,
                                const double *uene, const double *epsu, AlphaParams ap, double *adot,
                                double *adotu, bool f32) {
    GRID_STRIDE(p, n) {
        for (int c = 0; c < 3; ++c) {
            const double h = acch_r[3 * p + c];
            const double g1 = G * accg_r[3 * p + c];
            acch[3 * p + c] = h;
            accg1[3 * p + c] = g1;
            acc[3 * p + c] = h + g1 + accg2[3 * p + c];
        }
        udot[p] = udot_r[p];
        vsmx[p] = vsmx_r[p];
        const double df = diffu_r[p];
        diffu[p] = df;
        const double src = fmax(-divv[p] * (ap.amax - alph[p]), 0.0);
        // f32: the damping rate and conduction source in FP32 arithmetic
        const double tauinv = f32 ? (double)((0.25f * (float)KSRH * (float)vsnd[p]) / (float)ksr[p])
                                  : (0.25 * KSRH * vsnd[p]) / ksr[p];
        adot[p] = -(alph[p] - ap.amin) * tauinv + src;
        const double u = fmax(uene[p] - 0.0, 0.0);
        const double srcu = f32 ? (double)((float)ksr[p] / (float)KSRH * fabsf((float)df) / sqrtf((float)(u + *epsu)) *
                                           (float)fmax(ap.aumax - alphu[p], 0.0))
                                : ksr[p] / KSRH * fabs(df) / sqrt(u + *epsu) * fmax(ap.aumax - alphu[p], 0.0);
        adotu[p] = -(alphu[p] - ap.aumin) * tauinv + srcu;
    }
}

__global__ void finish_ksrmax(double *dsc, int mode) {
    // dsc[D_XC..D_MC] hold mass-weighted sums; dsc[D_R2], dsc[D_DN] the rho sums
    if (mode == 1 && dsc[D_DN] > 0.0) dsc[D_KSRMAX] = sqrt(dsc[D_R2] / dsc[D_DN]);
}

__global__ void com_divide(double *dsc) {
    const double m = dsc[D_MC];
    if (m > 0.0) {
        dsc[D_XC] /= m;
        dsc[D_YC] /= m;
        dsc[D_ZC] /= m;
    }
}

// calcTimestep's power-of-two adjustment, main.cpp:252-270
__global__ void update_dt(double *dsc, int *scal, double dt_max, double dt_min) {
    const double dtc = dsc[D_DTC];
    double dt = dsc[D_DT];
    const double t = dsc[D_TIME];
    if (dt > dtc) {
        while (dt > dtc) {
            dt *= 0.5;
            if (dt <= dt_min) {
                atomicOr(&scal[S_ERROR], E_DTMIN);
                break;
            }
        }
    } else if (2.0 * dt <= dtc && 2.0 * dt <= dt_max) {
        const double dt2 = 2.0 * dt;
        if (t - (double)(long long)(t / dt2) * dt2 == 0.0) dt *= 2.0;
    }
    dsc[D_DT] = dt;
}

// predict, hdr_hgas.hpp:646-657 (dnuc = 0, gcor3 = 0)
__global__ void predict(int n, const double *dsc, dbl4 *pos, dbl4 *vel, dbl4 *vel2, const double *acc,
                        double *uene, double *uene2, const double *udot, double *alph, double *alph2,
                        const double *adot, double *alphu, double *alphu2, const double *adotu) {
    const double dt = dsc[D_DT];
    GRID_STRIDE(p, n) {
        dbl4 x = pos[p];
        dbl4 v = vel[p];
        const double ax = acc[3 * p], ay = acc[3 * p + 1], az = acc[3 * p + 2];
        x.x = x.x + v.x * dt + 0.5 * ax * dt * dt;
        x.y = x.y + v.y * dt + 0.5 * ay * dt * dt;
        x.z = x.z + v.z * dt + 0.5 * az * dt * dt;
        pos[p] = x;
        vel2[p] = make_dbl4(v.x + 0.5 * ax * dt, v.y + 0.5 * ay * dt, v.z + 0.5 * az * dt, 0.0);
        vel[p] = make_dbl4(v.x + ax * dt, v.y + ay * dt, v.z + az * dt, 0.0);
        uene2[p] = uene[p] + 0.5 * udot[p] * dt;
        uene[p] = uene[p] + udot[p] * dt;
        alph2[p] = alph[p] + 0.5 * adot[p] * dt;
        alph[p] = alph[p] + adot[p] * dt;
        alphu2[p] = alphu[p] + 0.5 * adotu[p] * dt;
        alphu[p] = alphu[p] + adotu[p] * dt;
    }
}

// correct, hdr_hgas.hpp:659-665
__global__ void correct(int n, const double *dsc, dbl4 *vel, const dbl4 *vel2, const double *acc,
                        double *uene, const double *uene2, const double *udot, double *alph,
                        const double *alph2, const double *adot, double *alphu, const double *alphu2,
                        const double *adotu) {
    const double dt = dsc[D_DT];
    GRID_STRIDE(p, n) {
        const dbl4 v2 = vel2[p];
        vel[p] = make_dbl4(v2.x + 0.5 * acc[3 * p] * dt, v2.y + 0.5 * acc[3 * p + 1] * dt,
                           v2.z + 0.5 * acc[3 * p + 2] * dt, 0.0);
        uene[p] = uene2[p] + 0.5 * udot[p] * dt;
        alph[p] = alph2[p] + 0.5 * adot[p] * dt;
        alphu[p] = alphu2[p] + 0.5 * adotu[p] * dt;
    }
}

__global__ void advance_time(double *dsc) { dsc[D_TIME] += dsc[D_DT]; }

// dst (current order) from src (upload order): dst[p] = src[orig[p]]
__global__ void gather_field(int n, int width, const int *orig, const double *src, double *dst) {
    GRID_STRIDE(p, n) {
        const int q = orig[p];
        for (int c = 0; c < width; ++c) dst[(size_t)p * width + c] = src[(size_t)q * width + c];
    }
}

__global__ void scatter_field(int n, int width, const int *orig, const double *src, double *dst) {
    GRID_STRIDE(p, n) {
        const int q = orig[p];
        for (int c = 0; c < width; ++c) dst[(size_t)q * width + c] = src[(size_t)p * width + c];
    }
}

__global__ void field_from_dbl4(int n, const dbl4 *src, int comp, double *dst) {
    GRID_STRIDE(p, n) {
        const dbl4 v = src[p];
        if (comp < 0) {
            dst[3 * p] = v.x;
            dst[3 * p + 1] = v.y;
            dst[3 * p + 2] = v.z;
        } else {
            dst[p] = comp == 3 ? v.w : (comp == 0 ? v.x : (comp == 1 ? v.y : v.z));
        }
    }
}

template <class T>
__global__ void field_to_double(int n, const T *src, double *dst) {
    GRID_STRIDE(p, n) { dst[p] = (double)src[p]; }
}

__global__ void upload_pack(int n, const double *mass, const double *pos, const double *vel, dbl4 *opos,
                            dbl4 *ovel, dbl4 *ovel2) {
    GRID_STRIDE(p, n) {
        opos[p] = make_dbl4(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2], mass[p]);
        ovel[p] = make_dbl4(vel[3 * p], vel[3 * p + 1], vel[3 * p + 2], 0.0);
        ovel2[p] = ovel[p];
    }
}

__global__ void iota(int n, int *a) {
    GRID_STRIDE(p, n) { a[p] = p; }
}

__global__ void fill_double(int n, double *a, double v) {
    GRID_STRIDE(p, n) { a[p] = v; }
}

}  // namespace

// ======================================================================= system
// The buffers of one list builder: traversal tasks (per group count/offset,
// n + 1; per task (group, start node) and list count/offset, task_cap + 1),
// the chunk pool and the chunk ids of each task, the CUB scratch of its
// scans, the work items, and its scalars (sc: the system's for builder 0,
// own for builder 1, whose error bits are merged into the system's before
// its lists are used).
struct ListScratch {
    DevBuf<int> tcnt, toff, tlcnt, tloff;
    DevBuf<int2> tasks;
    int task_cap = 0;
    DevBuf<int> lpool, lchain;
    long long lpool_chunks = 0;
    int lchain_max = 0;
    DevBuf<char> cub;
    size_t cub_bytes = 0;
    DevBuf<WorkItem> items;
    DevBuf<int> own_sc;
    int *sc = nullptr;
    void release() {
        tcnt.release(); toff.release(); tlcnt.release(); tloff.release(); tasks.release();
        lpool.release(); lchain.release(); cub.release(); items.release(); own_sc.release();
    }
};

struct sph_system {
    sph_context *ctx = nullptr;
    int n = 0;
    sph_system_params prm;
    // persistent state (A) and permutation target (B)
    DevBuf<dbl4> pos[2], vel[2], vel2[2];
    DevBuf<long long> id[2];
    DevBuf<int> istar[2], orig[2];
    DevBuf<double> uene[2], uene2[2], alph[2], alph2[2], alphu[2], alphu2[2], ksr[2];
    // per-step state
    DevBuf<double> rs, dens, divv, rotv, grdh, pres, vsnd, bswt, eps2, udot, vsmx, diffu, pot, eta, adot,
        adotu;
    DevBuf<long long> np;
    DevBuf<dbl4> pe, h1, h2;
    DevBuf<double2> h3;
    DevBuf<double> acc, acch, accg1, accg2;
    DevBuf<double> t_dens, t_divv, t_rotv, t_grdh, t_ksr;
    DevBuf<long long> t_np;
    DevBuf<unsigned char> t_itr;
    DevBuf<double> r_acc, r_pot, r_eta, r_acch, r_accg, r_udot, r_vsmx, r_diffu;
    // tree
    DevBuf<uint64_t> keys[2];
    DevBuf<int> perm[2];
    DevBuf<int2> child;
    DevBuf<int> parent, first, count, visit;
    DevBuf<dbl4> mom;
    DevBuf<double> quad;          // 6 per node, quadrupole runs only
    DevBuf<float4> fq0, fq1;
    DevBuf<double> neps2;
    DevBuf<float4> flo, fhi, fmom, ptest;
    // FP32C double-float records (particles, hydro fields, tree monopoles)
    DevBuf<float4> f_phi, f_plo, f_vhi, f_vlo, f_g1, f_g2, f_g3, f_g4, f_shi, f_slo;
    // FP32C hydro: per particle the j indices of its marked pairs
    // (HYDRO_LIST_CAP per row), their number, and the rows that overflowed
    DevBuf<int> hl_list, hl_cnt;
    DevBuf<int2> hl_ovf;
    // re-walk index list (particles still iterating) and its per-walk segments
    DevBuf<int> uflag, uscan, ulist, a_sfirst, a_scount;
    // FP64 re-check queue of decision-ambiguous density results
    DevBuf<int> amb_i, amb_w;
    DevBuf<WorkItem> fitems;
    int amb_cap = 0;
    // per-warp neighbour lists of the density kernel (scratch)
    DevBuf<int> nbr;
    int nbr_warps = 0;
    DevBuf<double> w_csmax;   // per hydro walk: largest sound speed of its list
    // groups and walks
    DevBuf<int> gflag, groot, gscan, group_node, group_first, group_count;
    DevBuf<int> aflag, ascan, a_node, a_first, a_count;
    DevBuf<double> g_r, a_r;
    // lists per kind: 0 density (first walk), 1 hydro, 2 gravity,
    // 3 density re-walks (search radius expanded)
    DevBuf<int> lcnt[4], loff[4], jidx[4];
    // list builders: [0] density, re-walk and hydro lists, [1] gravity lists
    // (built on a second stream during graph replays, see force_body)
    ListScratch ls[2];
    DevBuf<int> roots;   // roots of the refit's bottom subtrees
    long long lcap[4] = {0, 0, 0, 0};
    int *walk_first[4] = {nullptr, nullptr, nullptr, nullptr};
    int *walk_count[4] = {nullptr, nullptr, nullptr, nullptr};
    int *walk_num[4] = {nullptr, nullptr, nullptr, nullptr};   // device count of walks
    // scalars
    DevBuf<int> scal;
    DevBuf<double> dscal, partial, box;
    DevBuf<long long> lscal;
    HostBuf<int> h_scal;
    HostBuf<double> h_dscal;
    HostBuf<long long> h_lscal;
    DevBuf<double> staging;
    DevBuf<double> an_buf;   // analysis scratch (4 n), allocated on first use
    DevBuf<double> h_guess;  // first guess of h of the last density evaluation
    // adjoint scratch, allocated on first use: accumulators, seeds, items
    DevBuf<double> adj_acc, adj_seed;
    DevBuf<sphadj::AdjItem> adj_items;
    DevBuf<int> adj_cnt, adj_off;
    // graph
    cudaGraphExec_t step_exec = nullptr;
    bool graph_valid = false;
    int graph_precision = -1;
    cudaGraphExec_t force_exec = nullptr;
    bool force_graph_valid = false;
    int force_graph_precision = -1;
    long long graph_kernels[2] = {-1, -1};   // kernel nodes of the force / step graph
    // phase events
    cudaEvent_t ev[16] = {nullptr};
    long long steps = 0;
    int last_status = 0;

    // capture of the re-walk loop body runs on body_stream (st_override)
    cudaStream_t st_override = nullptr;
    cudaStream_t body_stream = nullptr;
    // the gravity list build's stream in captured graphs, and the events that
    // fork it from and join it to the main stream
    cudaStream_t side_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool glist_forked = false;
    long long rewalk_kernels[2] = {0, 0};   // kernel nodes of the loop body (force / step graph)
    int capturing = -1;                     // graph being captured: 0 force, 1 step
    cudaStream_t st() const { return st_override ? st_override : ctx->stream; }
    Persist persist(int k) {
        Persist p;
        p.pos = pos[k].p; p.vel = vel[k].p; p.vel2 = vel2[k].p; p.id = id[k].p; p.istar = istar[k].p;
        p.orig = orig[k].p; p.uene = uene[k].p; p.uene2 = uene2[k].p; p.alph = alph[k].p;
        p.alph2 = alph2[k].p; p.alphu = alphu[k].p; p.alphu2 = alphu2[k].p; p.ksr = ksr[k].p;
        return p;
    }
    sphtree::Nodes nodes() {
        sphtree::Nodes t;
        t.child = child.p; t.parent = parent.p; t.first = first.p; t.count = count.p;
        t.mom = mom.p; t.eps2 = neps2.p; t.visit = visit.p;
        t.quad = quad.p; t.fq0 = fq0.p; t.fq1 = fq1.p;
        t.flo = flo.p; t.fhi = fhi.p; t.fmom = fmom.p; t.ptest = ptest.p;
        return t;
    }
};

namespace {

// Phase event k on stream st.  Inside a capture it becomes an external
// event-record node, so that every replay of the graph times its phases as
// well (sph_system_phase_times after a captured step or evaluation).
void phase_event(sph_system *s, int k, cudaStream_t st) {
    if (s->capturing >= 0)
        cudaEventRecordWithFlags(s->ev[k], st, cudaEventRecordExternal);
    else
        cudaEventRecord(s->ev[k], st);
}

int alloc_all(sph_system *s) {
    const size_t n = (size_t)s->n;
    const size_t nn = 2 * n;
    int e = 0;
    for (int k = 0; k < 2; ++k) {
        e |= s->pos[k].ensure(n) | s->vel[k].ensure(n) | s->vel2[k].ensure(n) | s->id[k].ensure(n);
        e |= s->istar[k].ensure(n) | s->orig[k].ensure(n) | s->uene[k].ensure(n) | s->uene2[k].ensure(n);
        e |= s->alph[k].ensure(n) | s->alph2[k].ensure(n) | s->alphu[k].ensure(n) | s->alphu2[k].ensure(n);
        e |= s->ksr[k].ensure(n) | s->keys[k].ensure(n) | s->perm[k].ensure(n);
    }
    DevBuf<double> *d1[] = {&s->rs, &s->dens, &s->divv, &s->rotv, &s->grdh, &s->pres, &s->vsnd, &s->bswt,
                            &s->eps2, &s->udot, &s->vsmx, &s->diffu, &s->pot, &s->eta, &s->adot, &s->adotu,
                            &s->t_dens, &s->t_divv, &s->t_rotv, &s->t_grdh, &s->t_ksr, &s->r_pot, &s->r_eta,
                            &s->r_udot, &s->r_vsmx, &s->r_diffu, &s->g_r, &s->a_r};
    for (auto *b : d1) e |= b->ensure(n);
    DevBuf<double> *d3[] = {&s->acc, &s->acch, &s->accg1, &s->accg2, &s->r_acc, &s->r_acch, &s->r_accg,
                            &s->staging};
    for (auto *b : d3) e |= b->ensure(3 * n);
    e |= s->np.ensure(n) | s->t_np.ensure(n) | s->t_itr.ensure(n);
    e |= s->pe.ensure(n) | s->h1.ensure(n) | s->h2.ensure(n) | s->h3.ensure(n);
    e |= s->child.ensure(n) | s->parent.ensure(nn) | s->first.ensure(nn) | s->count.ensure(nn);
    e |= s->visit.ensure(n) | s->mom.ensure(nn) | s->neps2.ensure(nn);
    if (s->prm.quadrupole) e |= s->quad.ensure(6 * nn) | s->fq0.ensure(nn) | s->fq1.ensure(nn);
    e |= s->flo.ensure(nn) | s->fhi.ensure(nn) | s->fmom.ensure(nn) | s->ptest.ensure(n);
    DevBuf<float4> *f1[] = {&s->f_phi, &s->f_plo, &s->f_vhi, &s->f_vlo, &s->f_g1, &s->f_g2, &s->f_g3, &s->f_g4};
    for (auto *b : f1) e |= b->ensure(n);
    e |= s->hl_list.ensure(n * sphk::HYDRO_LIST_CAP) | s->hl_cnt.ensure(n) | s->hl_ovf.ensure(n);
    e |= s->f_shi.ensure(nn) | s->f_slo.ensure(nn);
    e |= s->uflag.ensure(n) | s->uscan.ensure(n) | s->ulist.ensure(n) | s->a_sfirst.ensure(n) | s->a_scount.ensure(n);
    s->amb_cap = std::max<int>(1024, s->n / 16);
    e |= s->amb_i.ensure(s->amb_cap) | s->amb_w.ensure(s->amb_cap) | s->fitems.ensure(s->amb_cap);
    s->nbr_warps = std::max(s->ctx->grid[0][0], s->ctx->grid[0][1]) * PAIR_WARPS;
    e |= s->nbr.ensure((size_t)s->nbr_warps * NBR_CAP * 32) | s->w_csmax.ensure(n);
    DevBuf<int> *i1[] = {&s->gflag, &s->groot, &s->gscan, &s->group_node, &s->group_first, &s->group_count,
                         &s->aflag, &s->ascan, &s->a_node, &s->a_first, &s->a_count};
    for (auto *b : i1) e |= b->ensure(n);
    for (int k = 0; k < 4; ++k) e |= s->lcnt[k].ensure(n + 1) | s->loff[k].ensure(n + 1);
    e |= s->roots.ensure(n);
    e |= s->scal.ensure(S_NI) | s->dscal.ensure(D_NI) | s->lscal.ensure(L_NI);
    for (int k = 0; k < 2; ++k) {
        ListScratch &L = s->ls[k];
        e |= L.tcnt.ensure(n + 1) | L.toff.ensure(n + 1);
        L.task_cap = n / 16 + 4096;
        e |= L.tasks.ensure(L.task_cap) | L.tlcnt.ensure(L.task_cap + 1) | L.tloff.ensure(L.task_cap + 1);
        L.lchain_max = 64;
        L.lpool_chunks = std::min((long long)n * 24 / sphtree::LIST_CHUNK + L.task_cap + 1024, MAX_POOL_CHUNKS);
        e |= L.lpool.ensure((size_t)L.lpool_chunks * sphtree::LIST_CHUNK) |
             L.lchain.ensure((size_t)L.task_cap * L.lchain_max);
        e |= L.items.ensure(n);
        if (k == 1) e |= L.own_sc.ensure(S_NI);
        L.sc = k == 0 ? s->scal.p : L.own_sc.p;
    }
    e |= s->partial.ensure(RED_BLOCKS * MAX_RED + MAX_RED) | s->box.ensure(8);
    e |= s->h_scal.ensure(S_NI) | s->h_dscal.ensure(D_NI) | s->h_lscal.ensure(L_NI);
    e |= s->h_guess.ensure(n);
    // CUB scratch: radix sort of (uint64, int) pairs and exclusive sums over n ints
    size_t b1 = 0, b2 = 0;
    cub::DoubleBuffer<uint64_t> kb(s->keys[0].p, s->keys[1].p);
    cub::DoubleBuffer<int> vb(s->perm[0].p, s->perm[1].p);
    cub::DeviceRadixSort::SortPairs(nullptr, b1, kb, vb, s->n, 0, 63);
    cub::DeviceScan::ExclusiveSum(nullptr, b2, s->gflag.p, s->gscan.p, std::max(s->n, s->ls[0].task_cap) + 1);
    s->ls[0].cub_bytes = std::max(b1, b2);
    s->ls[1].cub_bytes = b2;
    for (int k = 0; k < 2; ++k) e |= s->ls[k].cub.ensure(s->ls[k].cub_bytes);
    // the first density walk covers every group, in group order
    s->walk_first[0] = s->group_first.p; s->walk_count[0] = s->group_count.p; s->walk_num[0] = s->scal.p + S_NGROUPS;
    s->walk_first[3] = s->a_first.p; s->walk_count[3] = s->a_count.p; s->walk_num[3] = s->scal.p + S_NACTIVE;
    s->walk_first[1] = s->group_first.p; s->walk_count[1] = s->group_count.p; s->walk_num[1] = s->scal.p + S_NGROUPS;
    s->walk_first[2] = s->group_first.p; s->walk_count[2] = s->group_count.p; s->walk_num[2] = s->scal.p + S_NGROUPS;
    return e;
}

#define CUDA_TRY(x)                                                   \
    do {                                                              \
        cudaError_t e__ = (x);                                        \
        if (e__ != cudaSuccess) return sphrt::cuda_error(s->ctx, e__, #x); \
    } while (0)

int exclusive_scan(sph_system *s, const int *in, int *out, int count = -1, int builder = 0) {
    ListScratch &L = s->ls[builder];
    size_t bytes = L.cub_bytes;
    CUDA_TRY(cub::DeviceScan::ExclusiveSum(L.cub.p, bytes, in, out, count < 0 ? s->n : count, s->st()));
    return SPH_OK;
}

template <class F>
void reduce(sph_system *s, F f, double *out) {
    reduce_stage1<F><<<RED_BLOCKS, RED_THREADS, 0, s->st()>>>(s->n, f, s->partial.p);
    reduce_stage2<F><<<1, 32 * F::K, 0, s->st()>>>(s->partial.p, RED_BLOCKS, out);
}

// Morton sort + permutation + radix tree + refit + groups.
// Bottom-up refit of the node data (after the tree build, and again when h
// changed).  Boxes, moments, centres of mass and quadrupoles depend only on
// positions and masses: the refit after a change of h alone (full = false)
// recomputes just the nodes' largest h and softening.
int refit_tree(sph_system *s, bool full = true) {
    const int n = s->n;
    cudaStream_t st = s->st();
    sphtree::Nodes t = s->nodes();
    CUDA_TRY(cudaMemsetAsync(s->visit.p, 0, sizeof(int) * (size_t)std::max(n - 1, 1), st));
    if (!full) {
        sphtree::refit_bottom_h<<<s->ctx->sm_count * 8, sphtree::REFIT_B, 0, st>>>(
            s->ksr[0].p, s->eps2.p, n, t, s->roots.p, s->scal.p + S_NROOTS);
        sphtree::refit_top_h<<<s->ctx->sm_count * 2, 256, 0, st>>>(n, t, s->roots.p, s->scal.p + S_NROOTS);
        sphtree::normalise_eps2<<<grid_for(n), 256, 0, st>>>(n, t);
        return SPH_OK;
    }
    if (s->prm.quadrupole) {
        sphtree::refit_bottom<true><<<s->ctx->sm_count * 8, sphtree::REFIT_B, 0, st>>>(
            s->pos[0].p, s->ksr[0].p, s->eps2.p, n, t, s->roots.p, s->scal.p + S_NROOTS, s->box.p);
        sphtree::refit_top<true><<<s->ctx->sm_count * 2, 256, 0, st>>>(n, t, s->roots.p, s->scal.p + S_NROOTS,
                                                                      s->box.p);
    } else {
        sphtree::refit_bottom<false><<<s->ctx->sm_count * 8, sphtree::REFIT_B, 0, st>>>(
            s->pos[0].p, s->ksr[0].p, s->eps2.p, n, t, s->roots.p, s->scal.p + S_NROOTS, s->box.p);
        sphtree::refit_top<false><<<s->ctx->sm_count * 2, 256, 0, st>>>(n, t, s->roots.p, s->scal.p + S_NROOTS,
                                                                       s->box.p);
    }
    sphtree::normalise_nodes<<<grid_for(n), 256, 0, st>>>(n, t, s->box.p, s->prm.quadrupole != 0);
    return SPH_OK;
}

int build_tree(sph_system *s) {
    int r0 = SPH_OK;
    const int n = s->n;
    cudaStream_t st = s->st();
    phase_event(s, EV_TREE_B, st);
    bbox_stage1<<<RED_BLOCKS, RED_THREADS, 0, st>>>(s->pos[0].p, n, s->partial.p);
    bbox_stage2<<<1, 32 * 6, 0, st>>>(s->partial.p, RED_BLOCKS, s->box.p);
    sphtree::morton_keys<<<grid_for(n), 256, 0, st>>>(s->pos[0].p, n, s->box.p, s->keys[0].p, s->perm[0].p);
    cub::DoubleBuffer<uint64_t> kb(s->keys[0].p, s->keys[1].p);
    cub::DoubleBuffer<int> vb(s->perm[0].p, s->perm[1].p);
    size_t bytes = s->ls[0].cub_bytes;
    CUDA_TRY(cub::DeviceRadixSort::SortPairs(s->ls[0].cub.p, bytes, kb, vb, n, 0, 63, st));
    const uint64_t *keys = kb.Current();
    const int *idx = vb.Current();
    permute<<<grid_for(n), 256, 0, st>>>(n, idx, s->persist(0), s->persist(1));
    // copy back so that the persistent arrays stay at fixed addresses (graph replay)
    const size_t nb = (size_t)n;
    CUDA_TRY(cudaMemcpyAsync(s->pos[0].p, s->pos[1].p, nb * sizeof(dbl4), cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->vel[0].p, s->vel[1].p, nb * sizeof(dbl4), cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->vel2[0].p, s->vel2[1].p, nb * sizeof(dbl4), cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->id[0].p, s->id[1].p, nb * sizeof(long long), cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->istar[0].p, s->istar[1].p, nb * sizeof(int), cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->orig[0].p, s->orig[1].p, nb * sizeof(int), cudaMemcpyDeviceToDevice, st));
    DevBuf<double> *dd[][2] = {{&s->uene[0], &s->uene[1]}, {&s->uene2[0], &s->uene2[1]},
                               {&s->alph[0], &s->alph[1]}, {&s->alph2[0], &s->alph2[1]},
                               {&s->alphu[0], &s->alphu[1]}, {&s->alphu2[0], &s->alphu2[1]},
                               {&s->ksr[0], &s->ksr[1]}};
    for (auto &d : dd)
        CUDA_TRY(cudaMemcpyAsync(d[0]->p, d[1]->p, nb * sizeof(double), cudaMemcpyDeviceToDevice, st));
    sphtree::Nodes t = s->nodes();
    sphtree::build_radix_tree<<<grid_for(n), 256, 0, st>>>(keys, n, t);
    set_int<<<1, 1, 0, st>>>(s->scal.p + S_NROOTS, 0);
    sphtree::mark_subtrees<<<grid_for(2LL * n - 1), 256, 0, st>>>(t, n, s->roots.p, s->scal.p + S_NROOTS);
    eps2_from_h<<<grid_for(n), 256, 0, st>>>(n, s->ksr[0].p, s->eps2.p);
    r0 = refit_tree(s);
    if (r0) return r0;
    // groups
    CUDA_TRY(cudaMemsetAsync(s->gflag.p, 0, sizeof(int) * nb, st));
    sphtree::mark_groups<<<grid_for(2LL * n - 1), 256, 0, st>>>(t, n, s->prm.n_group, s->gflag.p, s->groot.p);
    int r = exclusive_scan(s, s->gflag.p, s->gscan.p);
    if (r) return r;
    compact_groups<<<grid_for(n), 256, 0, st>>>(n, s->gflag.p, s->gscan.p, s->groot.p, t, s->group_node.p,
                                                s->group_first.p, s->group_count.p, s->scal.p);
    phase_event(s, EV_TREE_E, st);
    return SPH_OK;
}

// Grows the task buffers (eager evaluations only) and the CUB scratch that
// scans them.
int grow_tasks(sph_system *s, ListScratch &L, int cap) {
    int e = L.tasks.ensure(cap) | L.tlcnt.ensure((size_t)cap + 1) | L.tloff.ensure((size_t)cap + 1) |
            L.lchain.ensure((size_t)cap * L.lchain_max);
    if (e) return sphrt::set_error(s->ctx, SPH_ERR_CUDA, "task allocation of %d entries failed", cap);
    L.task_cap = cap;
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, L.tlcnt.p, L.tloff.p, cap + 1);
    if (b > L.cub_bytes) {
        if (L.cub.ensure(b)) return sphrt::set_error(s->ctx, SPH_ERR_CUDA, "CUB scratch allocation failed");
        L.cub_bytes = b;
    }
    s->graph_valid = false;
    s->force_graph_valid = false;
    return SPH_OK;
}

void launch_tasks(int mode, bool write, int grid, const sphtree::ListArgs &a, int *cnt, const int *off, int2 *tasks,
                  int cap, cudaStream_t st) {
    const int th = sphtree::TRAV_WARPS * 32;
    if (mode == sphtree::GATHER) {
        if (write) sphtree::list_tasks<sphtree::GATHER, true><<<grid, th, 0, st>>>(a, cnt, off, tasks, cap);
        else sphtree::list_tasks<sphtree::GATHER, false><<<grid, th, 0, st>>>(a, cnt, off, tasks, cap);
    } else if (mode == sphtree::SYMMETRIC) {
        if (write) sphtree::list_tasks<sphtree::SYMMETRIC, true><<<grid, th, 0, st>>>(a, cnt, off, tasks, cap);
        else sphtree::list_tasks<sphtree::SYMMETRIC, false><<<grid, th, 0, st>>>(a, cnt, off, tasks, cap);
    } else {
        if (write) sphtree::list_tasks<sphtree::GRAVITY, true><<<grid, th, 0, st>>>(a, cnt, off, tasks, cap);
        else sphtree::list_tasks<sphtree::GRAVITY, false><<<grid, th, 0, st>>>(a, cnt, off, tasks, cap);
    }
}

// the chunk pass of the list traversal (sphtree::PASS_CHUNK)
void launch_lists(int mode, int grid, const sphtree::ListArgs &a, cudaStream_t st) {
    const int th = sphtree::TRAV_WARPS * 32;
    if (mode == sphtree::GATHER)
        sphtree::build_lists<sphtree::GATHER, sphtree::PASS_CHUNK><<<grid, th, 0, st>>>(a);
    else if (mode == sphtree::SYMMETRIC)
        sphtree::build_lists<sphtree::SYMMETRIC, sphtree::PASS_CHUNK><<<grid, th, 0, st>>>(a);
    else
        sphtree::build_lists<sphtree::GRAVITY, sphtree::PASS_CHUNK><<<grid, th, 0, st>>>(a);
}

__global__ void pool_usage(int *scal) {
    atomicMax(&scal[S_POOLMAX], scal[S_POOL]);
}

// Builds the lists of `kind` over the walks (group nodes + radii) and the
// matching work items.  In eager mode (no capture) the list capacity grows to
// the counted total first.
int build_lists_and_items(sph_system *s, int kind, const int *walk_node, const double *walk_r, bool eager,
                          long long *pairs, const int *item_first = nullptr, const int *item_count = nullptr,
                          int chunk = 32) {
    const int n = s->n;
    cudaStream_t st = s->st();
    const int builder = kind == 2 ? 1 : 0;
    ListScratch &L = s->ls[builder];
    int *sc = L.sc;
    sphtree::ListArgs a{};
    a.t = s->nodes();
    a.n = n;
    a.root = 0;
    a.box = s->box.p;
    a.n_groups = s->walk_num[kind];
    a.group_node = walk_node;
    a.r_group = walk_r;
    a.n_leaf = s->prm.n_leaf;
    a.inv_theta2 = (float)(1.0 / (s->prm.theta * s->prm.theta));
    a.error = sc + S_ERROR;
    const int tgrid = s->ctx->sm_count * 8;
    const int mode = (kind == 0 || kind == 3) ? sphtree::GATHER : (kind == 1 ? sphtree::SYMMETRIC : sphtree::GRAVITY);
    // 1. traversal tasks per group (count, scan, grow in eager mode, write)
    CUDA_TRY(cudaMemsetAsync(L.tcnt.p, 0, sizeof(int) * (size_t)(n + 1), st));
    launch_tasks(mode, false, tgrid, a, L.tcnt.p, L.toff.p, L.tasks.p, L.task_cap, st);
    int r = exclusive_scan(s, L.tcnt.p, L.toff.p, n + 1, builder);
    if (r) return r;
    if (eager) {
        int nt = 0;
        CUDA_TRY(cudaMemcpyAsync(&nt, L.toff.p + n, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if (nt + nt / 4 > L.task_cap) {
            r = grow_tasks(s, L, nt + nt / 2 + 1024);
            if (r) return r;
        }
    }
    task_total<<<1, 1, 0, st>>>(n, L.toff.p, L.task_cap, sc);
    launch_tasks(mode, true, tgrid, a, L.tcnt.p, L.toff.p, L.tasks.p, L.task_cap, st);
    // 2. list lengths per task, offsets per task and per group
    a.tasks = L.tasks.p;
    a.n_tasks = sc + S_NTASKS;
    a.count_out = L.tlcnt.p;
    a.offset = L.tloff.p;
    a.pool_next = sc + S_POOL;
    a.pool_error = sc + S_POOLERR;
    a.task_queue = sc + S_TQUEUE;
    // one traversal: counts per task and the entries into pool chunks; in
    // eager mode the pool and the chains grow until they hold the lists with
    // a quarter of headroom (graph replays cannot allocate).  A pool that
    // held this traversal's lists but lacks headroom grows only after
    // copy_lists has read it (growing frees the old buffer).
    long long pool_grow_to = 0;
    for (;;) {
        a.pool = L.lpool.p;
        a.pool_chunks = L.lpool_chunks;
        a.chain = L.lchain.p;
        a.chain_max = L.lchain_max;
        CUDA_TRY(cudaMemsetAsync(L.tlcnt.p, 0, sizeof(int) * (size_t)(L.task_cap + 1), st));
        CUDA_TRY(cudaMemsetAsync(sc + S_POOL, 0, 3 * sizeof(int), st));   // pool, pool error, task queue
        launch_lists(mode, tgrid, a, st);
        pool_usage<<<1, 1, 0, st>>>(sc);
        if (!eager) break;
        int pu[2];
        CUDA_TRY(cudaMemcpyAsync(pu, sc + S_POOL, sizeof(pu), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        const long long used = pu[0];
        const bool redo = pu[1] != 0;
        if (!redo && used + used / 4 <= L.lpool_chunks) break;
        if (redo && used > MAX_POOL_CHUNKS)
            return sphrt::set_error(s->ctx, SPH_ERR_CAPACITY,
                                    "the interaction lists need %lld chunks of %d entries, more than 32-bit list "
                                    "offsets address (smoothing lengths far beyond the particle spacing?)",
                                    used, sphtree::LIST_CHUNK);
        if (used + used / 4 > L.lpool_chunks && L.lpool_chunks < MAX_POOL_CHUNKS) {
            const long long want = std::min(used + used / 2 + 1024, MAX_POOL_CHUNKS);
            if (!redo) {
                pool_grow_to = want;   // this traversal's chunks are still in the pool
            } else {
                if (L.lpool.ensure((size_t)want * sphtree::LIST_CHUNK))
                    return sphrt::set_error(s->ctx, SPH_ERR_CUDA, "list pool allocation of %lld chunks failed",
                                            want);
                L.lpool_chunks = std::min((long long)(L.lpool.cap / sphtree::LIST_CHUNK), MAX_POOL_CHUNKS);
            }
        }
        if (pu[1] & 2) {
            L.lchain_max *= 2;
            if (L.lchain.ensure((size_t)L.task_cap * L.lchain_max))
                return sphrt::set_error(s->ctx, SPH_ERR_CUDA, "list chain allocation failed");
        }
        s->graph_valid = false;
        s->force_graph_valid = false;
        if (!redo) break;   // grown for headroom only: this traversal is complete
    }
    r = exclusive_scan(s, L.tlcnt.p, L.tloff.p, L.task_cap + 1, builder);
    if (r) return r;
    sphtree::group_lists<<<grid_for(n + 1), 256, 0, st>>>(n, s->walk_num[kind], L.toff.p, L.tloff.p,
                                                         L.task_cap, s->loff[kind].p, s->lcnt[kind].p);
    const int lslot = kind == 0 ? L_LIST_D : (kind == 1 ? L_LIST_H : (kind == 2 ? L_LIST_G : L_LIST_R));
    if (eager) {
        list_total<<<1, 1, 0, st>>>(n, s->lcnt[kind].p, s->loff[kind].p, (long long)1 << 62, sc, s->lscal.p, lslot);
        long long tot = 0;
        CUDA_TRY(cudaMemcpyAsync(&tot, s->lscal.p + lslot, sizeof(long long), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if (tot + tot / 4 + 1 > s->lcap[kind]) {   // keep a quarter of headroom for graph replays
            long long want = tot + tot / 2 + 1024;
            if (kind == 3) want = std::max(want, s->lcap[0]);   // re-walks may cover many walks
            if (s->jidx[kind].ensure((size_t)want))
                return sphrt::set_error(s->ctx, SPH_ERR_CUDA, "list allocation of %lld entries failed", tot);
            s->lcap[kind] = (long long)s->jidx[kind].cap;
            // both captured graphs hold the old buffer
            s->graph_valid = false;
            s->force_graph_valid = false;
        }
    }
    list_total<<<1, 1, 0, st>>>(n, s->lcnt[kind].p, s->loff[kind].p, s->lcap[kind], sc, s->lscal.p, lslot);
    // 3. the chunks to their list offsets
    a.j_idx = s->jidx[kind].p;
    a.capacity = s->lcap[kind];
    sphtree::copy_lists<<<s->ctx->sm_count * 8, sphtree::COPY_THREADS, 0, st>>>(a);
    if (pool_grow_to > 0) {
        // headroom for the next evaluations; the copy above has read the old
        // pool (freeing it waits for the device)
        CUDA_TRY(cudaStreamSynchronize(st));
        if (L.lpool.ensure((size_t)pool_grow_to * sphtree::LIST_CHUNK))
            return sphrt::set_error(s->ctx, SPH_ERR_CUDA, "list pool allocation of %lld chunks failed", pool_grow_to);
        L.lpool_chunks = std::min((long long)(L.lpool.cap / sphtree::LIST_CHUNK), MAX_POOL_CHUNKS);
    }
    // work items
    const int *ifirst = item_first ? item_first : s->walk_first[kind];
    const int *icount = item_count ? item_count : s->walk_count[kind];
    // density and hydro walks with long lists are split (their pair loops
    // drop most of the list); gravity lists are uniform and kept whole
    const int split_nj = (kind == 2) ? (1 << 30) : (s->prm.item_split_nj > 0 ? s->prm.item_split_nj : ITEM_SPLIT_NJ);
    int *bkt = sc + S_BKT;
    CUDA_TRY(cudaMemsetAsync(bkt, 0, sizeof(int) * (2 * NBKT + 2), st));
    item_buckets<<<grid_for(n), 256, 0, st>>>(n, s->walk_num[kind], icount, s->lcnt[kind].p, chunk, split_nj, bkt);
    bucket_offsets<<<1, 32, 0, st>>>(bkt, kind == 2 ? 0 : (s->prm.heavy_classes >= 0 ? s->prm.heavy_classes
                                                                                   : SPH_HEAVY_CLASSES));
    // light items in walk order: per-walk counts (the task arrays are free
    // again once the lists are built) and their scan
    light_counts<<<grid_for(n + 1), 256, 0, st>>>(n, s->walk_num[kind], icount, s->lcnt[kind].p, chunk, split_nj,
                                                  bkt, L.tcnt.p);
    r = exclusive_scan(s, L.tcnt.p, L.toff.p, n + 1, builder);
    if (r) return r;
    fill_items<<<grid_for(n), 256, 0, st>>>(n, s->walk_num[kind], ifirst, icount, chunk, split_nj, s->lcnt[kind].p,
                                            bkt, L.toff.p, L.items.p, sc + S_NITEMS, pairs);
    drop_items_on_overflow<<<1, 1, 0, st>>>(sc);
    return SPH_OK;
}

long long count_kernel_nodes(cudaGraph_t g);

// Walk `it` of the density iteration (hdr_density.hpp:372-415): 0 walks every
// particle on the kind-0 lists, >= 1 only the particles still iterating (rs
// expanded by 1.1) on kind-3 lists.  it < 0: a walk of the captured re-walk
// loop, whose index is kept on the device and which sets the loop's
// condition (cond) for the next walk.
int density_walk(sph_system *s, int it, bool eager, cudaGraphConditionalHandle cond = 0) {
    const int n = s->n;
    cudaStream_t st = s->st();
    sph_context *ctx = s->ctx;
    const bool f32 = ctx->prm.precision == SPH_PREC_FP32C;
    const int max_it = std::max(1, s->prm.max_density_iterations);
    const bool first = it == 0;
    DensOut tmp{s->t_dens.p, s->t_divv.p, s->t_rotv.p, s->t_grdh.p, s->t_ksr.p, s->t_np.p, s->t_itr.p};
    DensOut out{s->dens.p, s->divv.p, s->rotv.p, s->grdh.p, s->ksr[0].p, s->np.p, nullptr};
    CUDA_TRY(cudaMemsetAsync(s->aflag.p, 0, sizeof(int) * (size_t)n, st));
    group_rs_max<<<ctx->sm_count * 8, 256, 0, st>>>(s->scal.p, s->group_first.p, s->group_count.p, s->rs.p,
                                                     s->g_r.p, s->aflag.p);
    int r = exclusive_scan(s, s->aflag.p, s->ascan.p);
    if (r) return r;
    compact_active<<<grid_for(n), 256, 0, st>>>(n, s->scal.p, s->aflag.p, s->ascan.p, s->group_node.p,
                                                s->group_first.p, s->group_count.p, s->g_r.p, s->a_node.p,
                                                s->a_first.p, s->a_count.p, s->a_r.p, s->scal.p);
    // i-particles: only those still iterating (all of them in the first walk)
    iterating_flags<<<grid_for(n), 256, 0, st>>>(n, s->rs.p, s->uflag.p);
    r = exclusive_scan(s, s->uflag.p, s->uscan.p);
    if (r) return r;
    scatter_list<<<grid_for(n), 256, 0, st>>>(n, s->uflag.p, s->uscan.p, s->ulist.p);
    walk_segments<<<grid_for(n), 256, 0, st>>>(n, s->scal.p, s->a_first.p, s->a_count.p, s->uflag.p,
                                               s->uscan.p, s->a_sfirst.p, s->a_scount.p);
    if (!first) rewalk_small<<<1, 1, 0, st>>>(n, s->uflag.p, s->uscan.p, s->scal.p);
    const int kind = first ? 0 : 3;
    r = build_lists_and_items(s, kind, s->a_node.p, s->a_r.p, eager, s->lscal.p + (first ? L_PAIRS_D1 : L_PAIRS_D),
                              s->a_sfirst.p, s->a_scount.p, first ? 32 : 8);
    if (r) return r;
    CUDA_TRY(cudaMemsetAsync(s->scal.p + S_QUEUE, 0, sizeof(int), st));
    sphk::DensityArgs a{};
    a.n_eval = first ? reinterpret_cast<unsigned long long *>(s->lscal.p + L_EVAL_D1) : nullptr;
    a.n_pass = first ? reinterpret_cast<unsigned long long *>(s->lscal.p + L_DLISTED) : nullptr;
    const bool lists = s->prm.density_list_slack > 0.0f;
    a.nbr = lists ? s->nbr.p : nullptr;
    a.nbr_cap = NBR_CAP;
    a.nbr_warps = s->nbr_warps;
    a.nbr_slack = lists ? s->prm.density_list_slack : 1.0f;
    a.i_pm = s->pos[0].p; a.i_vel = s->vel[0].p; a.i_id = s->id[0].p; a.i_ksr = s->ksr[0].p;
    a.i_rs = s->rs.p;
    a.j_pm = s->pos[0].p; a.j_vel = s->vel[0].p; a.j_id = s->id[0].p;
    a.items = s->ls[0].items.p; a.n_items = 0; a.n_items_dev = s->scal.p + S_NITEMS;
    a.j_off = s->loff[kind].p; a.j_idx = s->jidx[kind].p; a.queue = s->scal.p + S_QUEUE;
    a.i_list = s->ulist.p;
    a.fi = sphk::F32Part{s->f_phi.p, s->f_plo.p, s->f_vhi.p, s->f_vlo.p};
    a.fj = a.fi;
    a.o_dens = tmp.dens; a.o_divv = tmp.divv; a.o_rotv = tmp.rotv; a.o_grdh = tmp.grdh; a.o_ksr = tmp.ksr;
    a.o_np = tmp.np; a.o_itr = tmp.itr;
    a.eta_ksrh = ctx->prm.eta * KSRH;
    a.ksr_max = ctx->prm.ksr_max > 0.0 ? ctx->prm.ksr_max : std::numeric_limits<double>::infinity();
    a.ksr_max_dev = (s->prm.ksr_max_mode == 1) ? s->dscal.p + D_KSRMAX : nullptr;
    a.amb_count = f32 ? s->scal.p + S_AMB : nullptr;
    a.amb_i = s->amb_i.p;
    a.amb_w = s->amb_w.p;
    a.amb_cap = s->amb_cap;
    a.amb_tol = sphrt::AMB_TOL;
    if (f32) CUDA_TRY(cudaMemsetAsync(s->scal.p + S_AMB, 0, sizeof(int), st));
    if (first) phase_event(s, EV_DENSK_B, st);
    if (!first) drop_items_if_small<<<1, 1, 0, st>>>(s->scal.p);
    sphrt::launch_density(a, ctx->prm.precision, ctx->grid[0][ctx->prm.precision == SPH_PREC_FP64], st);
    if (!first) {
        // few iterating particles: a block per walk instead (see density_rewalk_blocks)
        const int rg = ctx->sm_count * 4;
        const sphk::RewalkBounds bnd{n, s->lcap[kind], s->scal.p + S_ERROR, E_LISTCAP | E_STACK, E_BOUNDS};
        if (f32)
            sphk::density_rewalk_blocks<false><<<rg, sphk::REWALK_THREADS, 0, st>>>(
                a, s->scal.p + S_NACTIVE, s->a_sfirst.p, s->a_scount.p, s->scal.p + S_SMALL, bnd);
        else
            sphk::density_rewalk_blocks<true><<<rg, sphk::REWALK_THREADS, 0, st>>>(
                a, s->scal.p + S_NACTIVE, s->a_sfirst.p, s->a_scount.p, s->scal.p + S_SMALL, bnd);
    }
    if (first) phase_event(s, EV_DENSK_E, st);
    if (f32) {
        // FP64 recomputation of decision-ambiguous particles (same lists)
        sphk::make_fixup_items<<<8, 256, 0, st>>>(s->scal.p + S_AMB, s->amb_w.p, s->amb_cap, s->fitems.p,
                                                  s->scal.p + S_NFIX);
        accumulate_int<<<1, 1, 0, st>>>(s->scal.p + S_AMB, s->scal.p + S_AMBTOT);
        CUDA_TRY(cudaMemsetAsync(s->scal.p + S_QUEUE, 0, sizeof(int), st));
        sphk::DensityArgs f = a;
        f.n_eval = nullptr;
        f.n_pass = nullptr;
        f.nbr = nullptr;
        f.items = s->fitems.p;
        f.n_items_dev = s->scal.p + S_NFIX;
        f.i_list = s->amb_i.p;
        f.amb_count = nullptr;
        sphrt::launch_density(f, SPH_PREC_FP64, ctx->grid[0][1], st);
    }
    commit_density<<<grid_for(n), 256, 0, st>>>(n, s->rs.p, tmp, out, s->scal.p);
    if (it >= 0)
        iteration_end<<<1, 1, 0, st>>>(s->scal.p, max_it, it);
    else
        iteration_end_loop<<<1, 1, 0, st>>>(s->scal.p, max_it, cond);
    return SPH_OK;
}

// In a captured graph the re-walks (walks 1 .. max_it-1) form one
// conditional while-node whose body is a re-walk: it runs only as often as
// particles still iterate, instead of max_it - 1 captured walks that mostly
// find nothing to do.  Returns 1 if the graph could not take the node (the
// caller then captures the walks unrolled).
int capture_rewalk_loop(sph_system *s, int max_it, int *r_out) {
    cudaStream_t st = s->st();
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    if (!s->body_stream || cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess ||
        cs != cudaStreamCaptureStatusActive)
        return 1;
    cudaGraphConditionalHandle h;
    if (cudaGraphConditionalHandleCreate(&h, g, 0, 0) != cudaSuccess) return 1;
    rewalk_start<<<1, 1, 0, st>>>(s->scal.p, max_it, h);
    *r_out = SPH_OK;
    auto fail = [&](cudaError_t e, const char *what) {
        *r_out = sphrt::cuda_error(s->ctx, e, what);
        return 0;
    };
    cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd);
    if (e != cudaSuccess) return fail(e, "cudaStreamGetCaptureInfo");
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &p);
    if (e != cudaSuccess) return fail(e, "cudaGraphAddNode (re-walk loop)");
    cudaGraph_t body = p.conditional.phGraph_out[0];
    e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return fail(e, "cudaStreamUpdateCaptureDependencies");
    e = cudaStreamBeginCaptureToGraph(s->body_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail(e, "cudaStreamBeginCaptureToGraph");
    s->st_override = s->body_stream;
    const int r = density_walk(s, -1, false, h);
    s->st_override = nullptr;
    cudaGraph_t got = nullptr;
    e = cudaStreamEndCapture(s->body_stream, &got);
    if (r) {
        *r_out = r;
        return 0;
    }
    if (e != cudaSuccess) return fail(e, "cudaStreamEndCapture (re-walk loop)");
    if (s->capturing >= 0) s->rewalk_kernels[s->capturing] = count_kernel_nodes(body);
    return 0;
}

int density_phase(sph_system *s, bool eager) {
    const int n = s->n;
    cudaStream_t st = s->st();
    sph_context *ctx = s->ctx;
    phase_event(s, EV_DENS_B, st);
    const bool f32 = ctx->prm.precision == SPH_PREC_FP32C;
    if (f32)
        sphk::make_density_records<<<grid_for(n), 256, 0, st>>>(n, s->pos[0].p, s->vel[0].p, s->f_phi.p,
                                                                s->f_plo.p, s->f_vhi.p, s->f_vlo.p);
    init_rs<<<grid_for(n), 256, 0, st>>>(n, s->ksr[0].p, s->rs.p);
    // the first guess, kept for the derivative of this evaluation
    CUDA_TRY(cudaMemcpyAsync(s->h_guess.p, s->ksr[0].p, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    set_int<<<1, 1, 0, st>>>(s->scal.p + S_ITERS, 1);
    set_int<<<1, 1, 0, st>>>(s->scal.p + S_AMBTOT, 0);
    set_int<<<1, 1, 0, st>>>(s->scal.p + S_UNCONV, 0);
    const int max_it = std::max(1, s->prm.max_density_iterations);
    int r = density_walk(s, 0, eager);
    if (r) return r;
    if (eager) {
        // walk again while particles iterate (the host reads the walk count)
        for (int it = 1; it < max_it; ++it) {
            int walks = 0;
            CUDA_TRY(cudaMemcpyAsync(&walks, s->scal.p + S_ITERS, sizeof(int), cudaMemcpyDeviceToHost, st));
            CUDA_TRY(cudaStreamSynchronize(st));
            if (walks <= it) break;
            r = density_walk(s, it, true);
            if (r) return r;
        }
    } else if (max_it > 1) {
        if (s->capturing >= 0) s->rewalk_kernels[s->capturing] = 0;
        int rr = SPH_OK;
        if (capture_rewalk_loop(s, max_it, &rr)) {
            // no conditional node: every re-walk captured (they return at
            // once when no particle iterates)
            for (int it = 1; it < max_it; ++it) {
                r = density_walk(s, it, false);
                if (r) return r;
            }
        } else if (rr) {
            return rr;
        }
    }
    phase_event(s, EV_DENS_E, st);
    return SPH_OK;
}

// Error bits of list builder 1 into the system's.
__global__ void merge_errors(const int *from, int *scal) {
    if (from[S_ERROR]) atomicOr(&scal[S_ERROR], from[S_ERROR]);
}

// The gravity lists and work items (list builder 1).  They depend only on the
// tree (node boxes and centres of mass, which the refit after the density
// phase rewrites with the same values), so in a captured graph they are
// built on side_stream, forked after the tree build and joined before the
// gravity kernel, while the density phase runs on the main stream; eager
// evaluations build them in order on the main stream.
int gravity_lists(sph_system *s, bool eager) {
    const cudaStream_t prev = s->st_override;
    s->glist_forked = !eager && s->capturing >= 0 && s->side_stream != nullptr;
    if (s->glist_forked) {
        CUDA_TRY(cudaEventRecord(s->ev_fork, s->st()));
        CUDA_TRY(cudaStreamWaitEvent(s->side_stream, s->ev_fork, 0));
        s->st_override = s->side_stream;
    }
    const cudaStream_t st = s->st();
    phase_event(s, EV_GLIST_B, st);
    int r = SPH_OK;
    const cudaError_t em = cudaMemsetAsync(s->ls[1].sc, 0, sizeof(int) * S_NI, st);
    if (em != cudaSuccess) r = sphrt::cuda_error(s->ctx, em, "cudaMemsetAsync");
    if (!r) r = build_lists_and_items(s, 2, s->group_node.p, nullptr, eager, s->lscal.p + L_PAIRS_G);
    phase_event(s, EV_GLIST_E, st);
    if (s->glist_forked) {
        const cudaError_t ej = cudaEventRecord(s->ev_join, s->side_stream);
        s->st_override = prev;
        if (!r && ej != cudaSuccess) r = sphrt::cuda_error(s->ctx, ej, "cudaEventRecord");
    }
    return r;
}

int gravity_phase(sph_system *s) {
    const int n = s->n;
    cudaStream_t st = s->st();
    sph_context *ctx = s->ctx;
    if (s->glist_forked) CUDA_TRY(cudaStreamWaitEvent(st, s->ev_join, 0));
    s->glist_forked = false;
    merge_errors<<<1, 1, 0, st>>>(s->ls[1].sc, s->scal.p);
    if (ctx->prm.precision == SPH_PREC_FP32C) {
        sphk::make_gravity_records<<<grid_for(n), 256, 0, st>>>(n, s->pos[0].p, s->eps2.p, s->f_phi.p, s->f_plo.p);
        sphk::make_gravity_records<<<grid_for(2LL * n - 1), 256, 0, st>>>(2 * n - 1, s->mom.p, s->neps2.p,
                                                                          s->f_shi.p, s->f_slo.p);
    }
    CUDA_TRY(cudaMemsetAsync(s->scal.p + S_QUEUE, 0, sizeof(int), st));
    phase_event(s, EV_GK_B, st);
    sphk::GravityArgs a{};
    a.i_pe = s->pe.p;
    a.j_pm = s->pos[0].p; a.j_eps2 = s->eps2.p;
    a.s_pm = s->mom.p; a.s_eps2 = s->neps2.p;
    a.fi_phi = s->f_phi.p; a.fi_plo = s->f_plo.p; a.f_phi = s->f_phi.p; a.f_plo = s->f_plo.p;
    a.f_shi = s->f_shi.p; a.f_slo = s->f_slo.p;
    a.i_list = nullptr;
    a.n_split = n;
    a.items = s->ls[1].items.p; a.n_items = 0; a.n_items_dev = s->ls[1].sc + S_NITEMS;
    a.j_off = s->loff[2].p; a.j_idx = s->jidx[2].p; a.queue = s->scal.p + S_QUEUE;
    a.o_acc = s->r_acc.p; a.o_pot = s->r_pot.p; a.o_eta = s->r_eta.p;
    const bool q64 = s->prm.quadrupole && ctx->prm.precision == SPH_PREC_FP64;
    const bool q32 = s->prm.quadrupole && ctx->prm.precision != SPH_PREC_FP64;
    a.s_quad = q64 ? s->quad.p : nullptr;
    a.f_sq0 = q32 ? s->fq0.p : nullptr;
    a.f_sq1 = q32 ? s->fq1.p : nullptr;
    const int jt = (ctx->prm.precision == SPH_PREC_FP32C && s->prm.gravity_jtile == 64) ? 64 : 32;
    sphrt::launch_gravity(a, ctx->prm.precision,
                          jt == 64 ? ctx->grid_g64 : ctx->grid[2][ctx->prm.precision == SPH_PREC_FP64], st, jt);
    phase_event(s, EV_GK_E, st);
    gravity_writeback<<<grid_for(n), 256, 0, st>>>(n, s->prm.G, s->r_acc.p, s->r_pot.p, s->r_eta.p, s->ksr[0].p,
                                                   s->grdh.p, s->dens.p, s->accg2.p, s->pot.p, s->eta.p,
                                                   ctx->prm.precision == SPH_PREC_FP32C);
    return SPH_OK;
}

int hydro_phase(sph_system *s, bool eager) {
    const int n = s->n;
    cudaStream_t st = s->st();
    sph_context *ctx = s->ctx;
    phase_event(s, EV_HLIST_B, st);
    hydro_prep<<<grid_for(n), 256, 0, st>>>(n, s->ksr[0].p, s->pres.p, s->grdh.p, s->dens.p, s->bswt.p,
                                            s->vsnd.p, s->alph[0].p, s->alphu[0].p, s->uene[0].p, s->eta.p,
                                            s->h1.p, s->h2.p, s->h3.p, ctx->prm.precision == SPH_PREC_FP32C);
    if (ctx->prm.precision == SPH_PREC_FP32C)
        sphk::make_hydro_records<<<grid_for(n), 256, 0, st>>>(n, s->pos[0].p, s->vel[0].p, s->h1.p, s->h2.p,
                                                              s->h3.p, s->f_phi.p, s->f_plo.p, s->f_vhi.p,
                                                              s->f_vlo.p, s->f_g1.p, s->f_g2.p, s->f_g3.p,
                                                              s->f_g4.p);
    int r = build_lists_and_items(s, 1, s->group_node.p, nullptr, eager, s->lscal.p + L_PAIRS_H);
    if (r) return r;
    const bool f32 = ctx->prm.precision == SPH_PREC_FP32C;
    const bool skip = s->prm.hydro_signal_skip != 0;
    if (skip)
        walk_csmax<<<ctx->sm_count * 8, CSMAX_THREADS, 0, st>>>(s->walk_num[1], s->loff[1].p, s->jidx[1].p,
                                                     f32 ? s->f_g2.p : nullptr, s->h2.p, s->w_csmax.p, s->scal.p);
    CUDA_TRY(cudaMemsetAsync(s->scal.p + S_QUEUE, 0, sizeof(int), st));
    phase_event(s, EV_HK_B, st);
    sphk::HydroArgs a{};
    a.n_eval_near = reinterpret_cast<unsigned long long *>(s->lscal.p + L_EVAL_HN);
    a.n_eval_far = reinterpret_cast<unsigned long long *>(s->lscal.p + L_EVAL_HF);
    a.n_skip = reinterpret_cast<unsigned long long *>(s->lscal.p + L_HSKIP);
    a.n_mark = reinterpret_cast<unsigned long long *>(s->lscal.p + L_HMARK);
    a.walk_csmax = skip ? s->w_csmax.p : nullptr;
    a.sv_skip = skip ? 1 : 0;
    a.i_pm = s->pos[0].p; a.i_vel = s->vel[0].p; a.i_id = s->id[0].p;
    a.i_h1 = s->h1.p; a.i_h2 = s->h2.p; a.i_h3 = s->h3.p;
    a.j_pm = s->pos[0].p; a.j_vel = s->vel[0].p; a.j_id = s->id[0].p;
    a.j_h1 = s->h1.p; a.j_h2 = s->h2.p; a.j_h3 = s->h3.p;
    a.fi = sphk::F32Part{s->f_phi.p, s->f_plo.p, s->f_vhi.p, s->f_vlo.p};
    a.fj = a.fi;
    a.fi_g1 = s->f_g1.p; a.fi_g2 = s->f_g2.p; a.fi_g3 = s->f_g3.p;
    a.fj_g1 = s->f_g1.p; a.fj_g2 = s->f_g2.p; a.fj_g3 = s->f_g3.p;
    a.i_list = nullptr;
    a.items = s->ls[0].items.p; a.n_items = 0; a.n_items_dev = s->scal.p + S_NITEMS;
    a.j_off = s->loff[1].p; a.j_idx = s->jidx[1].p; a.queue = s->scal.p + S_QUEUE;
    a.o_acch = s->r_acch.p; a.o_accg = s->r_accg.p; a.o_udot = s->r_udot.p; a.o_vsmx = s->r_vsmx.p;
    a.o_diffu = s->r_diffu.p;
    a.fi_g4 = s->f_g4.p; a.fj_g4 = s->f_g4.p;
    a.df_list = s->hl_list.p; a.df_cap = sphk::HYDRO_LIST_CAP; a.df_cnt = s->hl_cnt.p;
    a.df_ovf = s->hl_ovf.p; a.df_novf = s->scal.p + S_HOVF; a.n_i = n;
    if (f32) {
        // rows of particles no work item reaches (a failed list build) stay
        // empty; the overflow queue starts empty
        CUDA_TRY(cudaMemsetAsync(s->hl_cnt.p, 0, sizeof(int) * (size_t)n, st));
        CUDA_TRY(cudaMemsetAsync(s->scal.p + S_HOVF, 0, sizeof(int), st));
    }
    sphrt::launch_hydro(a, ctx->prm.precision, ctx->grid[1][ctx->prm.precision == SPH_PREC_FP64], st,
                        ctx->grid_df, s->ev[EV_HK_MID], s->capturing >= 0);
    phase_event(s, EV_HK_E, st);
    AlphaParams ap{s->prm.alpha_max, s->prm.alpha_min, s->prm.alphu_max, s->prm.alphu_min};
    hydro_writeback<<<grid_for(n), 256, 0, st>>>(
        n, s->prm.G, s->r_acch.p, s->r_accg.p, s->r_udot.p, s->r_vsmx.p, s->r_diffu.p, s->acch.p, s->accg1.p,
        s->accg2.p, s->acc.p, s->udot.p, s->vsmx.p, s->diffu.p, s->divv.p, s->alph[0].p, s->alphu[0].p,
        s->vsnd.p, s->ksr[0].p, s->uene[0].p, s->dscal.p + D_EPSU, ap, s->adot.p, s->adotu.p,
        ctx->prm.precision == SPH_PREC_FP32C);
    return SPH_OK;
}

// calcSPHKernel (main.cpp:300-358).  energy: reduce the energies of the
// evaluated state (a step reduces them once, after its corrector, instead).
int force_body(sph_system *s, bool eager, bool energy = true) {
    const int n = s->n;
    cudaStream_t st = s->st();
    CUDA_TRY(cudaMemsetAsync(s->lscal.p, 0, sizeof(long long) * L_NI, st));
    CUDA_TRY(cudaMemsetAsync(s->scal.p + S_POOLMAX, 0, sizeof(int), st));
    int r = build_tree(s);
    if (r) return r;
    r = gravity_lists(s, eager);
    if (r) return r;
    r = density_phase(s, eager);
    if (r) return r;
    post_density<<<grid_for(n), 256, 0, st>>>(n, s->pos[0].p, s->dens.p, s->uene[0].p, s->divv.p, s->rotv.p,
                                              s->ksr[0].p, s->pres.p, s->vsnd.p, s->bswt.p, s->eps2.p, s->pe.p,
                                              s->ctx->prm.precision == SPH_PREC_FP32C);
    r = refit_tree(s, false);   // h (max h, softening) changed in the density phase
    if (r) return r;
    r = gravity_phase(s);
    if (r) return r;
    r = hydro_phase(s, eager);
    if (r) return r;
    if (s->prm.ksr_max_mode == 1) {
        Star0Com f0{};
        f0.pos = s->pos[0].p;
        f0.istar = s->istar[0].p;
        reduce(s, f0, s->dscal.p + D_XC);
        com_divide<<<1, 1, 0, st>>>(s->dscal.p);
        KsrMaxSums f1{};
        f1.pos = s->pos[0].p;
        f1.dens = s->dens.p;
        f1.xc = s->dscal.p + D_XC;
        reduce(s, f1, s->dscal.p + D_R2);
        finish_ksrmax<<<1, 1, 0, st>>>(s->dscal.p, 1);
    }
    if (energy) {
        Energy fe{};
        fe.pos = s->pos[0].p; fe.vel = s->vel[0].p; fe.uene = s->uene[0].p; fe.pot = s->pot.p;
        reduce(s, fe, s->dscal.p + D_EKIN);
    }
    phase_event(s, EV_END, st);
    return SPH_OK;
}

// loopSimulation body (hdr_hgas.hpp:1499-1540)
int step_body(sph_system *s, bool eager) {
    const int n = s->n;
    cudaStream_t st = s->st();
    TimestepMin ft{};
    ft.ksr = s->ksr[0].p; ft.vsmx = s->vsmx.p; ft.divv = s->divv.p; ft.accg1 = s->accg1.p;
    ft.accg2 = s->accg2.p; ft.c_dt = s->prm.c_dt; ft.dt_max = s->prm.dt_max;
    ft.f32 = s->ctx->prm.precision == SPH_PREC_FP32C;
    reduce(s, ft, s->dscal.p + D_DTC);
    update_dt<<<1, 1, 0, st>>>(s->dscal.p, s->scal.p, s->prm.dt_max, s->prm.dt_min);
    predict<<<grid_for(n), 256, 0, st>>>(n, s->dscal.p, s->pos[0].p, s->vel[0].p, s->vel2[0].p, s->acc.p,
                                         s->uene[0].p, s->uene2[0].p, s->udot.p, s->alph[0].p, s->alph2[0].p,
                                         s->adot.p, s->alphu[0].p, s->alphu2[0].p, s->adotu.p);
    int r = force_body(s, eager, false);
    if (r) return r;
    correct<<<grid_for(n), 256, 0, st>>>(n, s->dscal.p, s->vel[0].p, s->vel2[0].p, s->acc.p, s->uene[0].p,
                                         s->uene2[0].p, s->udot.p, s->alph[0].p, s->alph2[0].p, s->adot.p,
                                         s->alphu[0].p, s->alphu2[0].p, s->adotu.p);
    advance_time<<<1, 1, 0, st>>>(s->dscal.p);
    Energy fe{};
    fe.pos = s->pos[0].p; fe.vel = s->vel[0].p; fe.uene = s->uene[0].p; fe.pot = s->pot.p;
    reduce(s, fe, s->dscal.p + D_EKIN);
    return SPH_OK;
}

int check_errors(sph_system *s) {
    int sc[S_NI];
    CUDA_TRY(cudaMemcpyAsync(sc, s->scal.p, sizeof(int) * S_NI, cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaStreamSynchronize(s->st()));
    const int e = sc[S_ERROR];
    if (e & E_STACK) return sphrt::set_error(s->ctx, SPH_ERR_CAPACITY, "tree walk stack overflow");
    if (e & E_LISTCAP) return sphrt::set_error(s->ctx, SPH_ERR_CAPACITY, "interaction list capacity exceeded");
    if (e & E_NOTCONV)
        return sphrt::set_error(s->ctx, SPH_ERR_NOT_CONVERGED, "search radius still growing after %d walks",
                                s->prm.max_density_iterations);
    if (e & E_DTMIN) return sphrt::set_error(s->ctx, SPH_ERR_NOT_CONVERGED, "time step below dt_min");
    if (e & E_BOUNDS) return sphrt::set_error(s->ctx, SPH_ERR_STATE, "index out of range in a density re-walk");
    return SPH_OK;
}

// Before a call: the error bits collect every problem of the call's steps.
int clear_errors(sph_system *s) {
    CUDA_TRY(cudaMemsetAsync(s->scal.p + S_ERROR, 0, sizeof(int), s->st()));
    return SPH_OK;
}

// After a graph replay: lists that filled more than 80% of their capacity
// send the next call through an eager evaluation, which grows them (graph
// replays cannot allocate).
int check_headroom(sph_system *s) {
    long long lc[L_NI];
    CUDA_TRY(cudaMemcpyAsync(lc, s->lscal.p, sizeof(lc), cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaStreamSynchronize(s->st()));
    const int slot[4] = {L_LIST_D, L_LIST_H, L_LIST_G, L_LIST_R};
    for (int k = 0; k < 4; ++k)
        if (lc[slot[k]] * 5 > s->lcap[k] * 4) {
            s->graph_valid = false;
            s->force_graph_valid = false;
        }
    for (int k = 0; k < 2; ++k) {
        int pm = 0;
        CUDA_TRY(cudaMemcpyAsync(&pm, s->ls[k].sc + S_POOLMAX, sizeof(int), cudaMemcpyDeviceToHost, s->st()));
        CUDA_TRY(cudaStreamSynchronize(s->st()));
        if ((long long)pm * 5 > s->ls[k].lpool_chunks * 4) {
            s->graph_valid = false;
            s->force_graph_valid = false;
        }
    }
    return SPH_OK;
}

bool capacity_error(int r) { return r == SPH_ERR_CAPACITY; }

}  // namespace

// ============================================================== C ABI
extern "C" void sph_system_params_default(sph_system_params *p) {
    if (!p) return;
    p->n_group = 256;
    p->n_leaf = 8;
    p->theta = 0.5;
    p->G = 6.6738480e-8 / ((6.9599e10 * 1e-3) * (6.9599e10 * 1e-3) * (6.9599e10 * 1e-3) / (1.9891e33 * 1e-6));
    p->c_dt = 0.1;
    p->dt_max = 10.0;
    p->dt_min = 1e-16;
    p->alpha_max = 2.0;
    p->alpha_min = 0.1;
    p->alphu_max = 0.0;
    p->alphu_min = 0.0;
    p->ksr_max_mode = 1;
    p->max_density_iterations = 8;
    p->use_graph = 1;
    p->quadrupole = 0;
    p->item_split_nj = ITEM_SPLIT_NJ;
    p->heavy_classes = SPH_HEAVY_CLASSES;
    p->density_list_slack = NBR_SLACK;
    p->hydro_signal_skip = 1;
    p->gravity_jtile = 32;
}

// update_dt halves the step until it is below the limit or at dt_min: that
// loop ends only for a positive dt_min and a finite dt_max.
static bool dt_range_ok(const sph_system_params &p) {
    return p.dt_min > 0.0 && p.dt_max >= p.dt_min && p.dt_max < INFINITY;
}

extern "C" int sph_system_create(sph_context *ctx, int64_t n, const sph_system_params *p, sph_system **out) {
    if (!ctx || !out || n < 2 || n > (1LL << 30)) return SPH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    sph_system *s = new (std::nothrow) sph_system();
    if (!s) return SPH_ERR_CAPACITY;
    s->ctx = ctx;
    s->n = (int)n;
    if (p) s->prm = *p; else sph_system_params_default(&s->prm);
    if (s->prm.n_group < 1 || s->prm.n_leaf < 1 || s->prm.n_leaf > sphtree::MAX_LEAF || !(s->prm.theta > 0.0) ||
        s->prm.density_list_slack > MAX_NBR_SLACK || !dt_range_ok(s->prm) ||
        (s->prm.gravity_jtile != 32 && s->prm.gravity_jtile != 64)) {
        delete s;
        return SPH_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(ctx->prm.device);
    ctx->n_systems++;   // released by sph_system_destroy
    if (alloc_all(s)) {
        sph_system_destroy(s);
        return sphrt::set_error(ctx, SPH_ERR_CUDA, "system allocation for %lld particles failed", (long long)n);
    }
    for (int k = 0; k < EV_N; ++k) cudaEventCreate(&s->ev[k]);
    cudaStreamCreateWithFlags(&s->body_stream, cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&s->side_stream, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming);
    cudaMemset(s->scal.p, 0, sizeof(int) * S_NI);
    cudaMemset(s->dscal.p, 0, sizeof(double) * D_NI);
    if (s->prm.quadrupole) {   // leaves keep Q = 0 (the refit writes internal nodes only)
        cudaMemset(s->quad.p, 0, s->quad.cap * sizeof(double));
        cudaMemset(s->fq0.p, 0, s->fq0.cap * sizeof(float4));
        cudaMemset(s->fq1.p, 0, s->fq1.cap * sizeof(float4));
    }
    cudaMemset(s->lscal.p, 0, sizeof(long long) * L_NI);
    *out = s;
    return SPH_OK;
}

extern "C" int sph_system_destroy(sph_system *s) {
    if (!s) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    cudaStreamSynchronize(s->st());
    if (s->step_exec) cudaGraphExecDestroy(s->step_exec);
    if (s->force_exec) cudaGraphExecDestroy(s->force_exec);
    for (int k = 0; k < EV_N; ++k)
        if (s->ev[k]) cudaEventDestroy(s->ev[k]);
    if (s->body_stream) cudaStreamDestroy(s->body_stream);
    if (s->side_stream) cudaStreamDestroy(s->side_stream);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    for (int k = 0; k < 2; ++k) {
        s->pos[k].release(); s->vel[k].release(); s->vel2[k].release(); s->id[k].release();
        s->istar[k].release(); s->orig[k].release(); s->uene[k].release(); s->uene2[k].release();
        s->alph[k].release(); s->alph2[k].release(); s->alphu[k].release(); s->alphu2[k].release();
        s->ksr[k].release(); s->keys[k].release(); s->perm[k].release();
    }
    DevBuf<double> *d1[] = {&s->rs, &s->dens, &s->divv, &s->rotv, &s->grdh, &s->pres, &s->vsnd, &s->bswt,
                            &s->eps2, &s->udot, &s->vsmx, &s->diffu, &s->pot, &s->eta, &s->adot, &s->adotu,
                            &s->t_dens, &s->t_divv, &s->t_rotv, &s->t_grdh, &s->t_ksr, &s->r_pot, &s->r_eta,
                            &s->r_udot, &s->r_vsmx, &s->r_diffu, &s->g_r, &s->a_r, &s->acc, &s->acch,
                            &s->accg1, &s->accg2, &s->r_acc, &s->r_acch, &s->r_accg, &s->staging,
                            &s->neps2, &s->dscal, &s->partial, &s->box};
    for (auto *b : d1) b->release();
    s->np.release(); s->t_np.release(); s->t_itr.release(); s->pe.release(); s->h1.release();
    s->h2.release(); s->h3.release(); s->child.release(); s->parent.release(); s->first.release();
    s->count.release(); s->visit.release(); s->mom.release(); s->quad.release(); s->fq0.release();
    s->fq1.release();
    DevBuf<float4> *f1[] = {&s->flo, &s->fhi, &s->fmom, &s->ptest, &s->f_phi, &s->f_plo, &s->f_vhi, &s->f_vlo,
                            &s->f_g1, &s->f_g2, &s->f_g3, &s->f_g4, &s->f_shi, &s->f_slo};
    for (auto *b : f1) b->release();
    s->hl_list.release(); s->hl_cnt.release(); s->hl_ovf.release();
    s->uflag.release(); s->uscan.release(); s->ulist.release(); s->a_sfirst.release(); s->a_scount.release();
    s->amb_i.release(); s->amb_w.release(); s->fitems.release(); s->nbr.release(); s->w_csmax.release();
    DevBuf<int> *i1[] = {&s->gflag, &s->groot, &s->gscan, &s->group_node, &s->group_first, &s->group_count,
                         &s->aflag, &s->ascan, &s->a_node, &s->a_first, &s->a_count,
                         &s->scal};
    for (auto *b : i1) b->release();
    for (int k = 0; k < 4; ++k) {
        s->lcnt[k].release(); s->loff[k].release(); s->jidx[k].release();
        if (k == 0) {
            s->ls[0].release();
            s->ls[1].release();
            s->roots.release();
        }
    }
    s->lscal.release(); s->an_buf.release();
    s->h_scal.release(); s->h_dscal.release(); s->h_lscal.release();
    s->h_guess.release(); s->adj_acc.release(); s->adj_seed.release(); s->adj_items.release();
    s->adj_cnt.release(); s->adj_off.release();
    s->ctx->n_systems--;
    delete s;
    return SPH_OK;
}

extern "C" int sph_system_upload(sph_system *s, double t0, const int64_t *id, const int32_t *istar,
                                 const double *mass, const double *pos, const double *vel, const double *uene,
                                 const double *ksr, const double *alph, const double *alphu) {
    if (!s || !id || !mass || !pos || !vel || !uene || !ksr) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    const int n = s->n;
    const size_t nb = (size_t)n;
    cudaStream_t st = s->st();
    // staging holds 3n doubles; the four 1-D arrays go to per-step buffers first
    CUDA_TRY(cudaMemcpyAsync(s->r_acc.p, pos, 3 * nb * sizeof(double), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->staging.p, vel, 3 * nb * sizeof(double), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->r_pot.p, mass, nb * sizeof(double), cudaMemcpyHostToDevice, st));
    upload_pack<<<grid_for(n), 256, 0, st>>>(n, s->r_pot.p, s->r_acc.p, s->staging.p, s->pos[0].p,
                                             s->vel[0].p, s->vel2[0].p);
    CUDA_TRY(cudaMemcpyAsync(s->id[0].p, id, nb * sizeof(long long), cudaMemcpyHostToDevice, st));
    if (istar)
        CUDA_TRY(cudaMemcpyAsync(s->istar[0].p, istar, nb * sizeof(int), cudaMemcpyHostToDevice, st));
    else
        CUDA_TRY(cudaMemsetAsync(s->istar[0].p, 0, nb * sizeof(int), st));
    iota<<<grid_for(n), 256, 0, st>>>(n, s->orig[0].p);
    CUDA_TRY(cudaMemcpyAsync(s->uene[0].p, uene, nb * sizeof(double), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->uene2[0].p, uene, nb * sizeof(double), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->ksr[0].p, ksr, nb * sizeof(double), cudaMemcpyHostToDevice, st));
    if (alph) {
        CUDA_TRY(cudaMemcpyAsync(s->alph[0].p, alph, nb * sizeof(double), cudaMemcpyHostToDevice, st));
    } else {
        fill_double<<<grid_for(n), 256, 0, st>>>(n, s->alph[0].p, 1.0);
    }
    if (alphu) {
        CUDA_TRY(cudaMemcpyAsync(s->alphu[0].p, alphu, nb * sizeof(double), cudaMemcpyHostToDevice, st));
    } else {
        fill_double<<<grid_for(n), 256, 0, st>>>(n, s->alphu[0].p, 0.0);
    }
    CUDA_TRY(cudaMemcpyAsync(s->alph2[0].p, s->alph[0].p, nb * sizeof(double), cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->alphu2[0].p, s->alphu[0].p, nb * sizeof(double), cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaMemsetAsync(s->acc.p, 0, 3 * nb * sizeof(double), st));
    CUDA_TRY(cudaMemsetAsync(s->udot.p, 0, nb * sizeof(double), st));
    CUDA_TRY(cudaMemsetAsync(s->adot.p, 0, nb * sizeof(double), st));
    CUDA_TRY(cudaMemsetAsync(s->adotu.p, 0, nb * sizeof(double), st));
    // run parameters that the reference derives from the initial state:
    // Timestep = MaximumTimestep (hdr_hgas.hpp:1244), ksrmax = star separation
    // (hdr_hgas.hpp:1335), epsu = 1e-4 min u (hdr_hgas.hpp:961-970)
    double dh[D_NI];
    std::memset(dh, 0, sizeof(dh));
    dh[D_TIME] = t0;
    dh[D_DT] = s->prm.dt_max;
    CUDA_TRY(cudaMemcpyAsync(s->dscal.p, dh, sizeof(dh), cudaMemcpyHostToDevice, st));
    UeneMin fu{};
    fu.uene = s->uene[0].p;
    reduce(s, fu, s->dscal.p + D_EPSU);
    StarComs fc{};
    fc.pos = s->pos[0].p;
    fc.istar = s->istar[0].p;
    reduce(s, fc, s->box.p);
    upload_scalars<<<1, 1, 0, st>>>(s->box.p, s->dscal.p);
    CUDA_TRY(cudaStreamSynchronize(st));   // the caller's host arrays are free again
    s->steps = 0;
    return SPH_OK;
}

namespace {
// Number of kernel nodes of a captured graph (one launch each per replay).
long long count_kernel_nodes(cudaGraph_t g) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return -1;
    std::vector<cudaGraphNode_t> nodes(n);
    if (n && cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return -1;
    long long k = 0;
    for (size_t i = 0; i < n; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) != cudaSuccess) return -1;
        if (t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

int capture(sph_system *s, bool step, cudaGraphExec_t *exec) {
    cudaStream_t st = s->st();
    if (*exec) {
        cudaGraphExecDestroy(*exec);
        *exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    s->capturing = step ? 1 : 0;
    const int rc = step ? step_body(s, false) : force_body(s, false);
    s->capturing = -1;
    const cudaError_t ec = cudaStreamEndCapture(st, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ec != cudaSuccess) return sphrt::cuda_error(s->ctx, ec, "cudaStreamEndCapture");
    s->graph_kernels[step ? 1 : 0] = count_kernel_nodes(g);
    const cudaError_t ei = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return sphrt::cuda_error(s->ctx, ei, "cudaGraphInstantiate");
    return SPH_OK;
}
}  // namespace

extern "C" int sph_system_compute_forces(sph_system *s) {
    if (!s) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    int r = clear_errors(s);
    if (r) return r;
    if (s->force_graph_precision != s->ctx->prm.precision) s->force_graph_valid = false;
    if (s->prm.use_graph && s->force_graph_valid) {
        const cudaError_t e = cudaGraphLaunch(s->force_exec, s->st());
        if (e != cudaSuccess) return sphrt::cuda_error(s->ctx, e, "cudaGraphLaunch");
        r = check_errors(s);
        if (!r) r = check_headroom(s);
        if (capacity_error(r)) {
            // a list outgrew its buffer during the replay: the evaluation
            // only changes derived fields and h (which the density iteration
            // re-converges), so it is repeated eagerly with grown buffers
            s->graph_valid = false;
            s->force_graph_valid = false;
            r = clear_errors(s);
            if (r) return r;
        } else {
            s->last_status = r;
            return r;
        }
    }
    // eager evaluation (sizes the lists); the graph is captured afterwards
    r = force_body(s, true);
    if (!r) r = check_errors(s);
    if (!r && s->prm.use_graph) {
        r = capture(s, false, &s->force_exec);
        if (!r) {
            s->force_graph_valid = true;
            s->force_graph_precision = s->ctx->prm.precision;
        }
    }
    s->last_status = r;
    return r;
}

extern "C" int sph_system_graph_kernels(sph_system *s, int32_t step, int64_t *kernels) {
    if (!s || !kernels) return SPH_ERR_INVALID_ARGUMENT;
    const bool valid = step ? s->graph_valid : s->force_graph_valid;
    const long long k = s->graph_kernels[step ? 1 : 0];
    if (!valid || k < 0) return SPH_ERR_STATE;
    int walks = 1;
    CUDA_TRY(cudaMemcpyAsync(&walks, s->scal.p + S_ITERS, sizeof(int), cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaStreamSynchronize(s->st()));
    *kernels = k + s->rewalk_kernels[step ? 1 : 0] * (long long)std::max(0, walks - 1);
    return SPH_OK;
}

extern "C" int sph_system_set_params(sph_system *s, const sph_system_params *p) {
    if (!s || !p) return SPH_ERR_INVALID_ARGUMENT;
    if (p->n_group < 1 || p->n_leaf < 1 || p->n_leaf > sphtree::MAX_LEAF || !(p->theta > 0.0))
        return sphrt::set_error(s->ctx, SPH_ERR_INVALID_ARGUMENT, "n_group, n_leaf (1..%d) or theta out of range",
                                sphtree::MAX_LEAF);
    if (p->density_list_slack > MAX_NBR_SLACK)
        return sphrt::set_error(s->ctx, SPH_ERR_INVALID_ARGUMENT, "density_list_slack above %g", (double)MAX_NBR_SLACK);
    if (!dt_range_ok(*p))
        return sphrt::set_error(s->ctx, SPH_ERR_INVALID_ARGUMENT, "need 0 < dt_min <= dt_max < infinity");
    if (p->gravity_jtile != 32 && p->gravity_jtile != 64)
        return sphrt::set_error(s->ctx, SPH_ERR_INVALID_ARGUMENT, "gravity_jtile must be 32 or 64");
    if (p->quadrupole && !s->prm.quadrupole)
        return sphrt::set_error(s->ctx, SPH_ERR_INVALID_ARGUMENT,
                                "quadrupole needs a system created with it (node moment buffers)");
    const int use_graph = s->prm.use_graph;
    s->prm = *p;
    s->prm.use_graph = use_graph;
    s->graph_valid = false;
    s->force_graph_valid = false;
    return SPH_OK;
}

extern "C" int sph_system_set_graph(sph_system *s, int32_t use_graph) {
    if (!s) return SPH_ERR_INVALID_ARGUMENT;
    s->prm.use_graph = use_graph ? 1 : 0;
    return SPH_OK;
}

extern "C" int sph_system_step(sph_system *s, int32_t n_steps) {
    if (!s || n_steps < 0) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    cudaStream_t st = s->st();
    int r = clear_errors(s);
    if (r) return r;
    for (int k = 0; k < n_steps; ++k) {
        if (s->graph_precision != s->ctx->prm.precision) s->graph_valid = false;
        if (!s->prm.use_graph || !s->graph_valid) {
            // eager step (sizes lists, then the graph is captured for the next steps)
            r = step_body(s, true);
            if (!r) r = check_errors(s);
            if (!r && s->prm.use_graph) {
                r = capture(s, true, &s->step_exec);
                if (r) return r;
                s->graph_valid = true;
                s->graph_precision = s->ctx->prm.precision;
            }
        } else {
            CUDA_TRY(cudaGraphLaunch(s->step_exec, st));
            // errors of replayed steps accumulate; they are read at the end
            // of the call, or when the lists near their capacity
            if (k == n_steps - 1 || (k & 15) == 15) {
                r = check_errors(s);
                if (!r) r = check_headroom(s);
            }
        }
        s->steps++;
        s->last_status = r;
        if (r) {
            if (capacity_error(r)) {
                // the step ran on truncated lists: its state is not valid;
                // the next call is eager and grows the buffers
                s->graph_valid = false;
                s->force_graph_valid = false;
            }
            return r;
        }
    }
    return SPH_OK;
}

namespace {
// Returns the device array of a field (width 1 or 3) or materialises it into
// s->staging.
int field_ptr(sph_system *s, int field, const double **ptr, int *width) {
    const int n = s->n;
    cudaStream_t st = s->st();
    *width = 1;
    switch (field) {
        case SPH_F_POS: field_from_dbl4<<<grid_for(n), 256, 0, st>>>(n, s->pos[0].p, -1, s->staging.p); *ptr = s->staging.p; *width = 3; return 0;
        case SPH_F_VEL: field_from_dbl4<<<grid_for(n), 256, 0, st>>>(n, s->vel[0].p, -1, s->staging.p); *ptr = s->staging.p; *width = 3; return 0;
        case SPH_F_MASS: field_from_dbl4<<<grid_for(n), 256, 0, st>>>(n, s->pos[0].p, 3, s->staging.p); *ptr = s->staging.p; return 0;
        case SPH_F_ACC: *ptr = s->acc.p; *width = 3; return 0;
        case SPH_F_ACCH: *ptr = s->acch.p; *width = 3; return 0;
        case SPH_F_ACCG1: *ptr = s->accg1.p; *width = 3; return 0;
        case SPH_F_ACCG2: *ptr = s->accg2.p; *width = 3; return 0;
        case SPH_F_DENS: *ptr = s->dens.p; return 0;
        case SPH_F_PRES: *ptr = s->pres.p; return 0;
        case SPH_F_VSND: *ptr = s->vsnd.p; return 0;
        case SPH_F_KSR: *ptr = s->ksr[0].p; return 0;
        case SPH_F_DIVV: *ptr = s->divv.p; return 0;
        case SPH_F_ROTV: *ptr = s->rotv.p; return 0;
        case SPH_F_BSWT: *ptr = s->bswt.p; return 0;
        case SPH_F_GRDH: *ptr = s->grdh.p; return 0;
        case SPH_F_UENE: *ptr = s->uene[0].p; return 0;
        case SPH_F_UDOT: *ptr = s->udot.p; return 0;
        case SPH_F_ALPH: *ptr = s->alph[0].p; return 0;
        case SPH_F_ALPHU: *ptr = s->alphu[0].p; return 0;
        case SPH_F_POT: *ptr = s->pot.p; return 0;
        case SPH_F_ETA: *ptr = s->eta.p; return 0;
        case SPH_F_VSMX: *ptr = s->vsmx.p; return 0;
        case SPH_F_DIFFU: *ptr = s->diffu.p; return 0;
        case SPH_F_ADOT: *ptr = s->adot.p; return 0;
        case SPH_F_ADOTU: *ptr = s->adotu.p; return 0;
        case SPH_F_NP: field_to_double<long long><<<grid_for(n), 256, 0, st>>>(n, s->np.p, s->staging.p); *ptr = s->staging.p; return 0;
        case SPH_F_ID: field_to_double<long long><<<grid_for(n), 256, 0, st>>>(n, s->id[0].p, s->staging.p); *ptr = s->staging.p; return 0;
        case SPH_F_ISTAR: field_to_double<int><<<grid_for(n), 256, 0, st>>>(n, s->istar[0].p, s->staging.p); *ptr = s->staging.p; return 0;
        default: return 1;
    }
}
}  // namespace

extern "C" int sph_system_download(sph_system *s, int32_t field, double *out) {
    if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    const double *src = nullptr;
    int w = 1;
    if (field_ptr(s, field, &src, &w)) return SPH_ERR_INVALID_ARGUMENT;
    const int n = s->n;
    double *dst = (src == s->staging.p) ? s->r_acch.p : s->staging.p;
    scatter_field<<<grid_for(n), 256, 0, s->st()>>>(n, w, s->orig[0].p, src, dst);
    CUDA_TRY(cudaMemcpyAsync(out, dst, sizeof(double) * w * (size_t)n, cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaStreamSynchronize(s->st()));
    return SPH_OK;
}

namespace {
// Writable device array of a field (restart), or null.
double *field_target(sph_system *s, int field, int *width) {
    *width = 1;
    switch (field) {
        case SPH_F_ACC: *width = 3; return s->acc.p;
        case SPH_F_ACCH: *width = 3; return s->acch.p;
        case SPH_F_ACCG1: *width = 3; return s->accg1.p;
        case SPH_F_ACCG2: *width = 3; return s->accg2.p;
        case SPH_F_DENS: return s->dens.p;
        case SPH_F_PRES: return s->pres.p;
        case SPH_F_VSND: return s->vsnd.p;
        case SPH_F_KSR: return s->ksr[0].p;
        case SPH_F_DIVV: return s->divv.p;
        case SPH_F_ROTV: return s->rotv.p;
        case SPH_F_BSWT: return s->bswt.p;
        case SPH_F_GRDH: return s->grdh.p;
        case SPH_F_UENE: return s->uene[0].p;
        case SPH_F_UDOT: return s->udot.p;
        case SPH_F_ALPH: return s->alph[0].p;
        case SPH_F_ALPHU: return s->alphu[0].p;
        case SPH_F_POT: return s->pot.p;
        case SPH_F_ETA: return s->eta.p;
        case SPH_F_VSMX: return s->vsmx.p;
        case SPH_F_DIFFU: return s->diffu.p;
        case SPH_F_ADOT: return s->adot.p;
        case SPH_F_ADOTU: return s->adotu.p;
        default: return nullptr;
    }
}
}  // namespace

extern "C" int sph_system_set_field(sph_system *s, int32_t field, const double *data) {
    if (!s || !data) return SPH_ERR_INVALID_ARGUMENT;
    int w = 1;
    double *dst = field_target(s, field, &w);
    if (!dst) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    const int n = s->n;
    cudaStream_t st = s->st();
    // staging (3n doubles) receives the upload-order copy
    CUDA_TRY(cudaMemcpyAsync(s->staging.p, data, sizeof(double) * w * (size_t)n, cudaMemcpyHostToDevice, st));
    gather_field<<<grid_for(n), 256, 0, st>>>(n, w, s->orig[0].p, s->staging.p, dst);
    if (field == SPH_F_UENE)
        CUDA_TRY(cudaMemcpyAsync(s->uene2[0].p, dst, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    if (field == SPH_F_ALPH)
        CUDA_TRY(cudaMemcpyAsync(s->alph2[0].p, dst, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    if (field == SPH_F_ALPHU)
        CUDA_TRY(cudaMemcpyAsync(s->alphu2[0].p, dst, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return SPH_OK;
}

extern "C" int sph_system_get_clock(sph_system *s, double *time, double *dt, double *ksr_max, double *eps_u) {
    if (!s) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    double dc[D_NI];
    CUDA_TRY(cudaMemcpyAsync(dc, s->dscal.p, sizeof(dc), cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaStreamSynchronize(s->st()));
    if (time) *time = dc[D_TIME];
    if (dt) *dt = dc[D_DT];
    if (ksr_max) *ksr_max = dc[D_KSRMAX];
    if (eps_u) *eps_u = dc[D_EPSU];
    return SPH_OK;
}

extern "C" int sph_system_set_clock(sph_system *s, double time, double dt, double ksr_max, double eps_u) {
    if (!s) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    cudaStream_t st = s->st();
    const int slot[4] = {D_TIME, D_DT, D_KSRMAX, D_EPSU};
    const double val[4] = {time, dt, ksr_max, eps_u};
    for (int k = 0; k < 4; ++k)
        if (val[k] >= 0.0)
            CUDA_TRY(cudaMemcpyAsync(s->dscal.p + slot[k], &val[k], sizeof(double), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return SPH_OK;
}

extern "C" int sph_system_download_sorted(sph_system *s, int32_t field, double *out) {
    if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    const double *src = nullptr;
    int w = 1;
    if (field_ptr(s, field, &src, &w)) return SPH_ERR_INVALID_ARGUMENT;
    CUDA_TRY(cudaMemcpyAsync(out, src, sizeof(double) * w * (size_t)s->n, cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaStreamSynchronize(s->st()));
    return SPH_OK;
}

extern "C" int sph_system_get_stats(sph_system *s, sph_system_stats *o) {
    if (!s || !o) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    int sc[S_NI];
    double dc[D_NI];
    long long lc[L_NI];
    CUDA_TRY(cudaMemcpyAsync(sc, s->scal.p, sizeof(sc), cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaMemcpyAsync(dc, s->dscal.p, sizeof(dc), cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaMemcpyAsync(lc, s->lscal.p, sizeof(lc), cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaStreamSynchronize(s->st()));
    o->time = dc[D_TIME];
    o->dt = dc[D_DT];
    o->ksr_max = dc[D_KSRMAX];
    o->e_kin = dc[D_EKIN];
    o->e_thm = dc[D_ETHM];
    o->e_pot = dc[D_EPOT];
    o->e_tot = dc[D_EKIN] + dc[D_ETHM] + dc[D_EPOT];
    o->n_groups = sc[S_NGROUPS];
    o->density_iterations = sc[S_ITERS];
    o->pairs_density = lc[L_PAIRS_D] + lc[L_PAIRS_D1];
    o->pairs_density_first = lc[L_PAIRS_D1];
    o->pairs_hydro = lc[L_PAIRS_H];
    o->pairs_gravity = lc[L_PAIRS_G];
    o->list_density = lc[L_LIST_D];
    o->list_hydro = lc[L_LIST_H];
    o->list_gravity = lc[L_LIST_G];
    o->steps = s->steps;
    o->density_rechecked = sc[S_AMBTOT];
    o->evals_density_first = lc[L_EVAL_D1];
    o->evals_density_grad = lc[L_EVAL_DG1];
    o->evals_hydro_near = lc[L_EVAL_HN];
    o->evals_hydro_far = lc[L_EVAL_HF];
    o->density_list_passes = lc[L_DLISTED];
    o->density_sweep_passes = lc[L_DSWEPT];
    o->hydro_sv_tiles_skipped = lc[L_HSKIP];
    o->hydro_sv_tiles = lc[L_HTILES];
    o->hydro_pairs_marked = lc[L_HMARK];
    o->hydro_pair_slots = lc[L_HSLOTS];
    o->hydro_rows_overflowed = sc[S_HOVF];
    o->last_status = s->last_status;
    return SPH_OK;
}

extern "C" int sph_system_get_lists(sph_system *s, int32_t kind, int32_t *n_walk, int64_t *n_entries,
                                    int32_t *i_first, int32_t *i_count, int64_t *j_off, int32_t *j_idx) {
    if (!s || kind < 0 || kind > 3 || !n_walk || !n_entries) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    cudaStream_t st = s->st();
    int nw = 0;
    long long tot = 0;
    CUDA_TRY(cudaMemcpyAsync(&nw, s->walk_num[kind], sizeof(int), cudaMemcpyDeviceToHost, st));
    if (kind < 3) {
        const int lslot = kind == 0 ? L_LIST_D : (kind == 1 ? L_LIST_H : L_LIST_G);
        CUDA_TRY(cudaMemcpyAsync(&tot, s->lscal.p + lslot, sizeof(long long), cudaMemcpyDeviceToHost, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    if (kind == 3 && nw > 0) {   // the last re-walk: its entries end where its last walk's list ends
        int last[2] = {0, 0};
        CUDA_TRY(cudaMemcpyAsync(&last[0], s->loff[3].p + nw - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(&last[1], s->lcnt[3].p + nw - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        tot = (long long)last[0] + last[1];
    }
    *n_walk = nw;
    *n_entries = tot;
    if (!i_first || !i_count || !j_off || !j_idx) return SPH_OK;
    std::vector<int> off(nw > 0 ? nw : 1), cnt(nw > 0 ? nw : 1);
    if (nw > 0) {
        CUDA_TRY(cudaMemcpyAsync(i_first, s->walk_first[kind], sizeof(int) * nw, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(i_count, s->walk_count[kind], sizeof(int) * nw, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(off.data(), s->loff[kind].p, sizeof(int) * nw, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(cnt.data(), s->lcnt[kind].p, sizeof(int) * nw, cudaMemcpyDeviceToHost, st));
    }
    if (tot > 0)
        CUDA_TRY(cudaMemcpyAsync(j_idx, s->jidx[kind].p, sizeof(int) * (size_t)tot, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    for (int w = 0; w < nw; ++w) j_off[w] = off[w];
    j_off[nw] = nw > 0 ? (int64_t)off[nw - 1] + cnt[nw - 1] : 0;
    return SPH_OK;
}

extern "C" int sph_system_phase_times(sph_system *s, float *ms, int32_t n) {
    if (!s || !ms || n < 0) return -SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    const cudaError_t se = cudaEventSynchronize(s->ev[EV_END]);
    if (se != cudaSuccess) return -sphrt::cuda_error(s->ctx, se, "cudaEventSynchronize");
    const int pairs[10][2] = {{EV_TREE_B, EV_TREE_E}, {EV_DENS_B, EV_DENS_E}, {EV_DENSK_B, EV_DENSK_E},
                              {EV_GLIST_B, EV_GLIST_E}, {EV_GK_B, EV_GK_E},   {EV_HLIST_B, EV_HK_B},
                              {EV_HK_B, EV_HK_E},     {EV_TREE_B, EV_END},   {EV_HK_B, EV_HK_MID},
                              {EV_HK_MID, EV_HK_E}};
    int k = 0;
    for (; k < n && k < 10; ++k) {
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, s->ev[pairs[k][0]], s->ev[pairs[k][1]]) != cudaSuccess) {
            cudaGetLastError();
            t = -1.0f;
        }
        ms[k] = t;
    }
    return k;
}

extern "C" int sph_system_get_nodes(sph_system *s, double *mom, double *eps2) {
    if (!s || !mom || !eps2) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    const size_t nn = 2 * (size_t)s->n - 1;
    CUDA_TRY(cudaMemcpyAsync(mom, s->mom.p, sizeof(dbl4) * nn, cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaMemcpyAsync(eps2, s->neps2.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaStreamSynchronize(s->st()));
    return SPH_OK;
}

// ============================================================== analysis
namespace {
// distance of every particle of the set from (cx, cy, cz) (+inf outside the
// set) and its mass
__global__ void radii_from(int n, const dbl4 *pos, const int *istar, int star, double cx, double cy, double cz,
                           double *r, double *m) {
    GRID_STRIDE(p, n) {
        const dbl4 x = pos[p];
        const double dx = x.x - cx, dy = x.y - cy, dz = x.z - cz;
        r[p] = (star < 0 || istar[p] == star) ? sqrt(dx * dx + dy * dy + dz * dz) : INFINITY;
        m[p] = x.w;
    }
}

template <class F>
int reduce_to_host(sph_system *s, const F &f, double *out) {
    reduce(s, f, s->partial.p + RED_BLOCKS * MAX_RED);   // result slots after the partials
    CUDA_TRY(cudaMemcpyAsync(out, s->partial.p + RED_BLOCKS * MAX_RED, sizeof(double) * F::K,
                             cudaMemcpyDeviceToHost, s->st()));
    CUDA_TRY(cudaStreamSynchronize(s->st()));
    return SPH_OK;
}
}  // namespace

extern "C" int sph_system_center_of_gravity(sph_system *s, int32_t star, double *out) {
    if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    DensCentre f{};
    f.pos = s->pos[0].p; f.vel = s->vel[0].p; f.dens = s->dens.p; f.istar = s->istar[0].p; f.star = star;
    double a[7];
    const int r = reduce_to_host(s, f, a);
    if (r) return r;
    for (int k = 0; k < 6; ++k) out[k] = a[6] > 0.0 ? a[k] / a[6] : 0.0;
    out[6] = a[6];
    return SPH_OK;
}

extern "C" int sph_system_bound_mass(sph_system *s, int32_t star, const double *vel_ref, double *out) {
    if (!s || !vel_ref || !out) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    BoundMass f{};
    f.pos = s->pos[0].p; f.vel = s->vel[0].p; f.pot = s->pot.p; f.uene = s->uene[0].p; f.istar = s->istar[0].p;
    f.star = star; f.vx = vel_ref[0]; f.vy = vel_ref[1]; f.vz = vel_ref[2];
    return reduce_to_host(s, f, out);
}

extern "C" int sph_system_mass_within(sph_system *s, int32_t star, const double *center, double radius,
                                      double *out) {
    if (!s || !center || !out) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    MassWithin f{};
    f.pos = s->pos[0].p; f.istar = s->istar[0].p; f.star = star;
    f.cx = center[0]; f.cy = center[1]; f.cz = center[2]; f.r = radius;
    return reduce_to_host(s, f, out);
}

extern "C" int sph_system_radii_sorted(sph_system *s, int32_t star, const double *center, double *r_out,
                                       double *m_out, int64_t *count) {
    if (!s || !center || !count) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    const int n = s->n;
    cudaStream_t st = s->st();
    if (s->an_buf.ensure(4 * (size_t)n))
        return sphrt::set_error(s->ctx, SPH_ERR_CUDA, "analysis buffer allocation failed");
    double *r0 = s->an_buf.p, *m0 = r0 + n, *r1 = m0 + n, *m1 = r1 + n;
    radii_from<<<grid_for(n), 256, 0, st>>>(n, s->pos[0].p, s->istar[0].p, star, center[0], center[1], center[2],
                                            r0, m0);
    size_t bytes = 0;
    CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, bytes, r0, r1, m0, m1, n, 0, 64, st));
    if (bytes > s->ls[0].cub_bytes) {
        if (s->ls[0].cub.ensure(bytes)) return sphrt::set_error(s->ctx, SPH_ERR_CUDA, "CUB scratch allocation failed");
        s->ls[0].cub_bytes = bytes;
        s->graph_valid = false;
        s->force_graph_valid = false;
    }
    bytes = s->ls[0].cub_bytes;
    CUDA_TRY(cub::DeviceRadixSort::SortPairs(s->ls[0].cub.p, bytes, r0, r1, m0, m1, n, 0, 64, st));
    std::vector<double> rh(n);
    CUDA_TRY(cudaMemcpyAsync(rh.data(), r1, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    int64_t c = 0;
    while (c < n && rh[c] != INFINITY) ++c;
    *count = c;
    if (r_out) std::memcpy(r_out, rh.data(), sizeof(double) * (size_t)c);
    if (m_out) {
        CUDA_TRY(cudaMemcpyAsync(m_out, m1, sizeof(double) * (size_t)c, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    return SPH_OK;
}

// ---------------------------------------------------------------- derivative
// Leapfrog predictor alone (hdr_hgas.hpp:646-657) with the clock's current dt:
// with sph_system_compute_forces afterwards it reproduces the force evaluation
// of a step from that step's starting state, for sph_system_adjoint_forces.
extern "C" int sph_system_predict(sph_system *s) {
    if (!s) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->prm.device);
    const int n = s->n;
    cudaStream_t st = s->st();
    predict<<<grid_for(n), 256, 0, st>>>(n, s->dscal.p, s->pos[0].p, s->vel[0].p, s->vel2[0].p, s->acc.p,
                                         s->uene[0].p, s->uene2[0].p, s->udot.p, s->alph[0].p, s->alph2[0].p,
                                         s->adot.p, s->alphu[0].p, s->alphu2[0].p, s->adotu.p);
    CUDA_TRY(cudaStreamSynchronize(st));
    return SPH_OK;
}

// Vector-Jacobian product of the last force evaluation (adjoint.cuh).
// seed (host, upload order, 8n doubles): dL/d acc (3n), udot, adot, ksr (the
// final h), pot, dens.  grad (host, upload order, 9n doubles): dL/d position
// (3n), velocity (3n), internal energy, alpha, first guess of h.
extern "C" int sph_system_adjoint_forces(sph_system *s, const double *seed, double *grad) {
    if (!s || !seed || !grad) return SPH_ERR_INVALID_ARGUMENT;
    sph_context *ctx = s->ctx;
    cudaSetDevice(ctx->prm.device);
    const int n = s->n;
    cudaStream_t st = s->st();
    if (s->prm.quadrupole || s->prm.alphu_max != 0.0 || s->prm.alphu_min != 0.0 ||
        !(ctx->prm.ksr_max <= 0.0 && s->prm.ksr_max_mode == 0))
        return sphrt::set_error(ctx, SPH_ERR_STATE,
                                "the derivative covers monopole gravity, alpha_u fixed at 0 and no clamp of h "
                                "(ksr_max 0, ksr_max_mode 0)");
    int sc[S_NI];
    CUDA_TRY(cudaMemcpyAsync(sc, s->scal.p, sizeof(sc), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (sc[S_ITERS] != 1)
        return sphrt::set_error(ctx, SPH_ERR_STATE,
                                "the derivative needs a force evaluation with one density walk (got %d)", sc[S_ITERS]);
    const int ng = sc[S_NGROUPS];
    // scratch
    const int NA = 26;   // doubles per particle in the accumulators (+ 4 per node, 2n nodes)
    int e = s->adj_acc.ensure((size_t)NA * n + 8 * (size_t)n) | s->adj_seed.ensure(8 * (size_t)n + 9 * (size_t)n);
    e |= s->adj_cnt.ensure(n + 1) | s->adj_off.ensure(n + 1);
    if (e) return sphrt::set_error(ctx, SPH_ERR_CUDA, "adjoint scratch allocation failed");
    CUDA_TRY(cudaMemsetAsync(s->adj_acc.p, 0, sizeof(double) * ((size_t)NA * n + 8 * (size_t)n), st));
    // items: one warp per 32 particles of a group
    sphadj::adj_item_counts<<<grid_for(ng), 256, 0, st>>>(ng, s->group_count.p, s->adj_cnt.p);
    int r = exclusive_scan(s, s->adj_cnt.p, s->adj_off.p, ng);
    if (r) return r;
    int last[2];
    CUDA_TRY(cudaMemcpyAsync(&last[0], s->adj_off.p + ng - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&last[1], s->adj_cnt.p + ng - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    const int n_items = last[0] + last[1];
    if (s->adj_items.ensure(n_items)) return sphrt::set_error(ctx, SPH_ERR_CUDA, "adjoint item allocation failed");
    sphadj::adj_fill_items<<<grid_for(ng), 256, 0, st>>>(ng, s->group_first.p, s->group_count.p, s->adj_off.p,
                                                         s->adj_items.p);
    // seeds: host (upload order) -> device (sorted order)
    double *up = s->adj_seed.p, *sd = s->adj_seed.p + 8 * (size_t)n;
    CUDA_TRY(cudaMemcpyAsync(up, seed, sizeof(double) * 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    gather_field<<<grid_for(n), 256, 0, st>>>(n, 3, s->orig[0].p, up, sd);
    for (int k = 0; k < 5; ++k)
        gather_field<<<grid_for(n), 256, 0, st>>>(n, 1, s->orig[0].p, up + (3 + k) * (size_t)n,
                                                  sd + (3 + k) * (size_t)n);
    sphadj::AdjSeed sed{sd, sd + 3 * (size_t)n, sd + 4 * (size_t)n, sd + 5 * (size_t)n, sd + 6 * (size_t)n,
                        sd + 7 * (size_t)n};
    double *A = s->adj_acc.p;
    auto slot = [&](int k) { return A + (size_t)k * n; };
    sphadj::AdjAcc acc;
    acc.x = slot(0); acc.v = slot(3); acc.u = slot(6); acc.alph = slot(7); acc.h0 = slot(8);
    acc.h = slot(9); acc.rho = slot(10); acc.omega = slot(11); acc.divv = slot(12); acc.rotv = slot(13);
    acc.c = slot(14); acc.b = slot(15); acc.pc = slot(16); acc.eta = slot(17); acc.e2 = slot(18);
    acc.hinv = slot(19); acc.etas = slot(20); acc.bswt = slot(21);
    acc.node = slot(NA);   // 8n doubles: 4 per node
    sphadj::AdjState as;
    as.n = n;
    as.pos = s->pos[0].p; as.vel = s->vel[0].p; as.uene = s->uene[0].p; as.alph = s->alph[0].p;
    as.h0 = s->h_guess.p; as.h = s->ksr[0].p; as.dens = s->dens.p; as.grdh = s->grdh.p; as.divv = s->divv.p;
    as.rotv = s->rotv.p; as.pres = s->pres.p; as.vsnd = s->vsnd.p; as.bswt = s->bswt.p; as.eps2 = s->eps2.p;
    as.eta = s->eta.p; as.etas = s->r_eta.p;
    as.mom = s->mom.p; as.neps2 = s->neps2.p; as.parent = s->parent.p;
    as.d_off = s->loff[0].p; as.d_idx = s->jidx[0].p; as.h_off = s->loff[1].p; as.h_idx = s->jidx[1].p;
    as.g_off = s->loff[2].p; as.g_idx = s->jidx[2].p;
    as.G = s->prm.G; as.amax = s->prm.alpha_max; as.amin = s->prm.alpha_min; as.eta_ksrh = ctx->prm.eta * KSRH;
    const int eg = grid_for(n), wg = ctx->sm_count * 8;
    sphadj::adj_alpha<<<eg, 256, 0, st>>>(as, sed, acc);
    sphadj::adj_hydro<<<wg, 128, 0, st>>>(as, sed, acc, s->adj_items.p, n_items);
    sphadj::adj_hydro_prep<<<eg, 256, 0, st>>>(as, acc);
    sphadj::adj_gravity<<<wg, 128, 0, st>>>(as, sed, acc, s->adj_items.p, n_items);
    sphadj::adj_nodes<<<eg, 256, 0, st>>>(as, acc);
    sphadj::adj_switch<<<eg, 256, 0, st>>>(as, acc);
    sphadj::adj_density_grad<<<wg, 128, 0, st>>>(as, acc, s->adj_items.p, n_items);
    sphadj::adj_density_passes<<<wg, 128, 0, st>>>(as, acc, s->adj_items.p, n_items);
    // results: sorted -> upload order
    double *out = s->adj_seed.p;   // 9n doubles (the seeds are consumed)
    scatter_field<<<grid_for(n), 256, 0, st>>>(n, 3, s->orig[0].p, acc.x, out);
    scatter_field<<<grid_for(n), 256, 0, st>>>(n, 3, s->orig[0].p, acc.v, out + 3 * (size_t)n);
    scatter_field<<<grid_for(n), 256, 0, st>>>(n, 1, s->orig[0].p, acc.u, out + 6 * (size_t)n);
    scatter_field<<<grid_for(n), 256, 0, st>>>(n, 1, s->orig[0].p, acc.alph, out + 7 * (size_t)n);
    scatter_field<<<grid_for(n), 256, 0, st>>>(n, 1, s->orig[0].p, acc.h0, out + 8 * (size_t)n);
    CUDA_TRY(cudaMemcpyAsync(grad, out, sizeof(double) * 9 * (size_t)n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    const cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) return sphrt::cuda_error(ctx, ce, "adjoint kernels");
    return SPH_OK;
}
