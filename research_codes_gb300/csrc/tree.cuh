// tree.cuh — the GPU tree and interaction-list builder that calls the pair
// kernels in the device-resident path (the role FDPS plays for the reference:
// TreeForForceShort::Gather / ::Symmetry and TreeForForce<SEARCH_MODE_LONG>,
// main.cpp:377-397).
//
//   1. 63-bit Morton keys of the FP64 positions in the global bounding box;
//      CUB radix sort; particles permuted into key order.
//   2. Binary radix tree over the sorted keys (Karras 2012): internal nodes
//      0..n-2, leaf node n-1+p for particle p; one thread per internal node.
//   3. Bottom-up refit (one thread per leaf, second arrival combines): FP64
//      bounding box, particle range, max h, monopole (mass, centre of mass,
//      mass-weighted eps^2 as GravityMonopole, hdr_gravity.hpp:37-49).
//   4. i-groups ("walks"): maximal subtrees with <= n_group particles.
//   5. Lists, one warp per group, warp-cooperative batched-DFS traversal with a
//      shared-memory stack; two passes (count, then fill at scanned offsets)
//      so list order is deterministic:
//        gather    : j with dist(x_j, box_g) <= max_{i in g, unconverged} rs_i
//        symmetric : j with dist(x_j, box_g) <= max(max_{i in g} h_i, h_j)
//        gravity   : node accepted as a monopole when
//                    dist(box_g, com_node)^2 > (size_node / theta)^2,
//                    otherwise opened; unaccepted buckets of <= n_leaf
//                    particles enter as particles.  List index >= n means
//                    node (index - n).
#pragma once

#include <stdint.h>

#include "sph_device.cuh"

namespace sphtree {

using sphk::FULL;

constexpr int TRAV_WARPS = 4;
constexpr int STACK = 1024;   // per warp

struct Nodes {
    int2 *child;      // internal nodes: (left, right)
    int *parent;
    int *first;       // first particle (sorted index)
    int *count;
    dbl4 *lo;         // bbox min; w = max h in the subtree
    dbl4 *hi;         // bbox max; w = unused
    dbl4 *mom;        // centre of mass x, y, z; w = mass
    double *eps2;     // mass-weighted eps^2
    int *visit;       // refit arrival counters
    float4 *flo;      // FP32 traversal copies: lo (rounded down), w = max h (up)
    float4 *fhi;      // hi (rounded up), w = largest box side (up)
    float4 *fmom;     // centre of mass, mass
    float4 *ptest;    // per particle: position (nearest), h (rounded up)
};

// ---- 1. keys ------------------------------------------------------------
__device__ __forceinline__ uint64_t spread3(uint64_t v) {
    v &= 0x1fffffULL;
    v = (v | (v << 32)) & 0x1f00000000ffffULL;
    v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

// box[0..2] = min, box[3..5] = max (filled by a reduction kernel).
__global__ void morton_keys(const dbl4 *pos, int n, const double *box, uint64_t *keys, int *idx) {
    const double lx = box[0], ly = box[1], lz = box[2];
    double span = fmax(fmax(box[3] - lx, box[4] - ly), box[5] - lz);
    span = span > 0.0 ? span : 1.0;
    const double s = 2097151.0 / span;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const dbl4 x = pos[p];
        const uint64_t ix = (uint64_t)fmin(fmax((x.x - lx) * s, 0.0), 2097151.0);
        const uint64_t iy = (uint64_t)fmin(fmax((x.y - ly) * s, 0.0), 2097151.0);
        const uint64_t iz = (uint64_t)fmin(fmax((x.z - lz) * s, 0.0), 2097151.0);
        keys[p] = (spread3(ix) << 2) | (spread3(iy) << 1) | spread3(iz);
        idx[p] = p;
    }
}

// ---- 2. binary radix tree -------------------------------------------------
__device__ __forceinline__ int prefix_len(const uint64_t *k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = k[i], b = k[j];
    if (a == b) return 64 + __clz(i ^ j);
    return __clzll(a ^ b);
}

__global__ void build_radix_tree(const uint64_t *k, int n, Nodes t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (prefix_len(k, n, i, i + 1) - prefix_len(k, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = prefix_len(k, n, i, i - d);
    int lmax = 2;
    while (prefix_len(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int s = lmax >> 1; s >= 1; s >>= 1)
        if (prefix_len(k, n, i, i + (l + s) * d) > dmin) l += s;
    const int j = i + l * d;
    const int dnode = prefix_len(k, n, i, j);
    int s = 0;
    int step = l;
    do {
        step = (step + 1) >> 1;
        if (prefix_len(k, n, i, i + (s + step) * d) > dnode) s += step;
    } while (step > 1);
    const int gamma = i + s * d + min(d, 0);
    const int left = (min(i, j) == gamma) ? (n - 1 + gamma) : gamma;
    const int right = (max(i, j) == gamma + 1) ? (n - 1 + gamma + 1) : gamma + 1;
    t.child[i] = make_int2(left, right);
    t.parent[left] = i;
    t.parent[right] = i;
    if (i == 0) t.parent[0] = -1;
}

// ---- 3. refit ----------------------------------------------------------------
// L1-bypassing load: another thread (another SM) wrote the child nodes.
__device__ __forceinline__ dbl4 ldcg4(const dbl4 *p) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
    const double2 a = __ldcg(q), b = __ldcg(q + 1);
    return make_dbl4(a.x, a.y, b.x, b.y);
}

// FP32 copies of the node geometry for the traversal: boxes rounded outwards,
// h_max and size rounded up, so that FP32 tests are conservative.
__device__ __forceinline__ void write_fgeom(const Nodes &t, int node, const dbl4 &lo, const dbl4 &hi,
                                            const dbl4 &m) {
    const double size = fmax(fmax(hi.x - lo.x, hi.y - lo.y), hi.z - lo.z);
    t.flo[node] = make_float4(__double2float_rd(lo.x), __double2float_rd(lo.y), __double2float_rd(lo.z),
                              __double2float_ru(lo.w));
    t.fhi[node] = make_float4(__double2float_ru(hi.x), __double2float_ru(hi.y), __double2float_ru(hi.z),
                              __double2float_ru(size));
    t.fmom[node] = make_float4((float)m.x, (float)m.y, (float)m.z, (float)m.w);
}

__global__ void refit(const dbl4 *pos, const double *h, const double *eps2, int n, Nodes t) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int node = n - 1 + p;
    const dbl4 x = pos[p];
    t.first[node] = p;
    t.count[node] = 1;
    const dbl4 l0 = make_dbl4(x.x, x.y, x.z, h[p]);
    const dbl4 h0 = make_dbl4(x.x, x.y, x.z, 0.0);
    const dbl4 m0 = make_dbl4(x.x, x.y, x.z, x.w);
    t.lo[node] = l0;
    t.hi[node] = h0;
    t.mom[node] = m0;
    t.eps2[node] = eps2[p];
    write_fgeom(t, node, l0, h0, m0);
    t.ptest[p] = make_float4((float)x.x, (float)x.y, (float)x.z, __double2float_ru(h[p]));
    if (n == 1) return;
    node = t.parent[node];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&t.visit[node], 1) == 0) return;   // sibling not finished yet
        __threadfence();
        const int2 c = t.child[node];
        const dbl4 la = ldcg4(&t.lo[c.x]), lb = ldcg4(&t.lo[c.y]);
        const dbl4 ha = ldcg4(&t.hi[c.x]), hb = ldcg4(&t.hi[c.y]);
        const dbl4 ma = ldcg4(&t.mom[c.x]), mb = ldcg4(&t.mom[c.y]);
        const double ea = __ldcg(&t.eps2[c.x]), eb = __ldcg(&t.eps2[c.y]);
        const int ca = __ldcg(&t.count[c.x]), cb = __ldcg(&t.count[c.y]);
        const int fa = __ldcg(&t.first[c.x]);
        t.first[node] = fa;
        t.count[node] = ca + cb;
        const dbl4 lo = make_dbl4(fmin(la.x, lb.x), fmin(la.y, lb.y), fmin(la.z, lb.z), fmax(la.w, lb.w));
        const dbl4 hi = make_dbl4(fmax(ha.x, hb.x), fmax(ha.y, hb.y), fmax(ha.z, hb.z), 0.0);
        t.lo[node] = lo;
        t.hi[node] = hi;
        const double m = ma.w + mb.w;
        dbl4 mom;
        if (m > 0.0) {
            const double mi = 1.0 / m;
            mom = make_dbl4((ma.w * ma.x + mb.w * mb.x) * mi, (ma.w * ma.y + mb.w * mb.y) * mi,
                            (ma.w * ma.z + mb.w * mb.z) * mi, m);
            t.eps2[node] = (ma.w * ea + mb.w * eb) * mi;
        } else {
            mom = make_dbl4(0.5 * (lo.x + hi.x), 0.5 * (lo.y + hi.y), 0.5 * (lo.z + hi.z), 0.0);
            t.eps2[node] = 0.5 * (ea + eb);
        }
        t.mom[node] = mom;
        write_fgeom(t, node, lo, hi, mom);
        node = t.parent[node];
    }
}

// ---- 4. groups -------------------------------------------------------------
// flag[first particle of a group root] = 1, root_at[first] = node.
__global__ void mark_groups(Nodes t, int n, int n_group, int *flag, int *root_at) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= 2 * n - 1) return;
    const int c = t.count[v];
    const int p = t.parent[v];
    const int pc = (p >= 0) ? t.count[p] : 0x7fffffff;
    if (c <= n_group && pc > n_group) {
        const int f = t.first[v];
        flag[f] = 1;
        root_at[f] = v;
    }
}

// ---- 5. lists ---------------------------------------------------------------
enum ListMode { GATHER = 0, SYMMETRIC = 1, GRAVITY = 2 };

constexpr int CAND = 64;           // candidate buckets buffered per warp
constexpr int MAX_LEAF = 8;        // n_leaf limit (bucket expansion buffer)

struct ListArgs {
    Nodes t;
    int n;                  // particles
    int root;
    const double *box;      // global bounding box (min xyz, max xyz) of the step
    const int *n_groups;    // device count of groups to traverse
    const int *group_node;  // tree node of each group (indexed by position in this list)
    const double *r_group;  // gather: search radius of the group
    int n_leaf;             // <= MAX_LEAF
    float inv_theta2;
    // pass 1 writes counts, pass 2 fills at offsets
    int *count_out;
    const int *offset;      // exclusive scan of counts (fill pass)
    int *j_idx;
    long long capacity;     // entries available in j_idx
    int *error;             // bit 1: stack overflow, bit 2: capacity exceeded
};

__device__ __forceinline__ float box_box_d2f(const float4 &alo, const float4 &ahi, const float4 &blo,
                                             const float4 &bhi) {
    const float dx = fmaxf(0.0f, fmaxf(alo.x - bhi.x, blo.x - ahi.x));
    const float dy = fmaxf(0.0f, fmaxf(alo.y - bhi.y, blo.y - ahi.y));
    const float dz = fmaxf(0.0f, fmaxf(alo.z - bhi.z, blo.z - ahi.z));
    return dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ float point_box_d2f(float x, float y, float z, const float4 &lo, const float4 &hi) {
    const float dx = fmaxf(0.0f, fmaxf(lo.x - x, x - hi.x));
    const float dy = fmaxf(0.0f, fmaxf(lo.y - y, y - hi.y));
    const float dz = fmaxf(0.0f, fmaxf(lo.z - z, z - hi.z));
    return dx * dx + dy * dy + dz * dz;
}

// Search radius with FP32 safety margins: relative 2e-6 for the arithmetic,
// plus an absolute term covering the rounding of coordinates to FP32.
__device__ __forceinline__ float widen(float r, float slack) { return r * 1.000002f + slack; }

template <int MODE, bool FILL>
__global__ void __launch_bounds__(TRAV_WARPS * 32) build_lists(ListArgs a) {
    __shared__ int stack[TRAV_WARPS][STACK];
    __shared__ int cand[TRAV_WARPS][CAND];
    __shared__ int cpre[TRAV_WARPS][CAND + 1];
    __shared__ int pidx[TRAV_WARPS][CAND * MAX_LEAF];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int n_groups = *a.n_groups;
    const int warps = gridDim.x * TRAV_WARPS;
    // coordinates were rounded to FP32: |error| <= 2^-24 max|x| per axis
    const double cmax = fmax(fmax(fmax(fabs(a.box[0]), fabs(a.box[3])), fmax(fabs(a.box[1]), fabs(a.box[4]))),
                             fmax(fabs(a.box[2]), fabs(a.box[5])));
    const float slack = (float)(4.0e-7 * cmax);
    for (int g = blockIdx.x * TRAV_WARPS + wid; g < n_groups; g += warps) {
        const int gn = a.group_node[g];
        const float4 glo = a.t.flo[gn];
        const float4 ghi = a.t.fhi[gn];
        float rg = 0.0f;
        if (MODE == GATHER) rg = __double2float_ru(a.r_group[g]);
        if (MODE == SYMMETRIC) rg = glo.w;          // max h of the group (rounded up)
        long long out = FILL ? (long long)a.offset[g] : 0;
        int total = 0;
        int sp = 1, nc = 0;
        if (lane == 0) stack[wid][0] = a.root;
        __syncwarp();
        bool overflow = false;
        while (sp > 0 || nc > 0) {
            if (sp > 0) {
                const int take = min(sp, 32);
                const int node = (lane < take) ? stack[wid][sp - take + lane] : -1;
                sp -= take;
                __syncwarp();
                bool push = false, bucket = false, accept = false;
                int2 ch = make_int2(0, 0);
                if (node >= 0) {
                    const float4 lo = a.t.flo[node];
                    const float4 hi = a.t.fhi[node];
                    const bool leafish = (node >= a.n - 1) || a.t.count[node] <= a.n_leaf;
                    if (MODE == GRAVITY) {
                        const float4 m = a.t.fmom[node];
                        const float d2 = point_box_d2f(m.x, m.y, m.z, glo, ghi);
                        if (d2 > hi.w * hi.w * a.inv_theta2) accept = true;
                        else if (leafish) bucket = true;
                        else push = true;
                    } else {
                        const float r = widen(MODE == SYMMETRIC ? fmaxf(rg, lo.w) : rg, slack);
                        if (box_box_d2f(glo, ghi, lo, hi) <= r * r) {
                            if (leafish) bucket = true;
                            else push = true;
                        }
                    }
                    if (push) ch = a.t.child[node];
                }
                // children of opened nodes
                const unsigned pm = __ballot_sync(FULL, push);
                if (sp + 2 * __popc(pm) > STACK) {
                    overflow = true;
                } else {
                    if (push) {
                        const int pre = __popc(pm & lt_mask);
                        stack[wid][sp + 2 * pre] = ch.y;
                        stack[wid][sp + 2 * pre + 1] = ch.x;
                    }
                    sp += 2 * __popc(pm);
                }
                // accepted monopoles (gravity)
                if (MODE == GRAVITY) {
                    const unsigned am = __ballot_sync(FULL, accept);
                    if (FILL && accept) {
                        const long long w = out + __popc(am & lt_mask);
                        if (w < a.capacity) a.j_idx[w] = a.n + node;
                        else atomicOr(a.error, 2);
                    }
                    out += __popc(am);
                    total += __popc(am);
                }
                // particle buckets to test
                const unsigned bm = __ballot_sync(FULL, bucket);
                if (bucket) cand[wid][nc + __popc(bm & lt_mask)] = node;
                nc += __popc(bm);
                __syncwarp();
            }
            if (nc >= 32 || (sp == 0 && nc > 0) || (overflow && nc > 0)) {
                // expand the buffered buckets into particle indices, then test
                // 32 particles at a time
                const int c0 = (lane < nc) ? a.t.count[cand[wid][lane]] : 0;
                const int c1 = (lane + 32 < nc) ? a.t.count[cand[wid][lane + 32]] : 0;
                int inc0 = c0, inc1 = c1;
                for (int o = 1; o < 32; o <<= 1) {
                    const int v0 = __shfl_up_sync(FULL, inc0, o);
                    const int v1 = __shfl_up_sync(FULL, inc1, o);
                    if (lane >= o) {
                        inc0 += v0;
                        inc1 += v1;
                    }
                }
                const int tot0 = __shfl_sync(FULL, inc0, 31);
                const int base0 = inc0 - c0, base1 = tot0 + inc1 - c1;
                const int tot = tot0 + __shfl_sync(FULL, inc1, 31);
                if (lane < nc) {
                    const int f = a.t.first[cand[wid][lane]];
                    for (int k = 0; k < c0; ++k) pidx[wid][base0 + k] = f + k;
                }
                if (lane + 32 < nc) {
                    const int f = a.t.first[cand[wid][lane + 32]];
                    for (int k = 0; k < c1; ++k) pidx[wid][base1 + k] = f + k;
                }
                __syncwarp();
                for (int b = 0; b < tot; b += 32) {
                    const int p = (b + lane < tot) ? pidx[wid][b + lane] : -1;
                    bool ok = p >= 0;
                    if (ok && MODE != GRAVITY) {
                        const float4 x = a.t.ptest[p];
                        const float r = widen(MODE == SYMMETRIC ? fmaxf(rg, x.w) : rg, slack);
                        ok = point_box_d2f(x.x, x.y, x.z, glo, ghi) <= r * r;
                    }
                    const unsigned om = __ballot_sync(FULL, ok);
                    if (FILL && ok) {
                        const long long w = out + __popc(om & lt_mask);
                        if (w < a.capacity) a.j_idx[w] = p;
                        else atomicOr(a.error, 2);
                    }
                    out += __popc(om);
                    total += __popc(om);
                }
                nc = 0;
                __syncwarp();
            }
            if (overflow) break;
        }
        if (overflow && lane == 0) atomicOr(a.error, 1);
        if (!FILL && lane == 0) a.count_out[g] = total;
    }
}

}  // namespace sphtree
