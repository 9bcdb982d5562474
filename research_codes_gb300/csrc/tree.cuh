// tree.cuh — the GPU tree and interaction-list builder that calls the pair
// kernels in the device-resident path (the role FDPS plays for the reference:
// TreeForForceShort::Gather / ::Symmetry and TreeForForce<SEARCH_MODE_LONG>,
// main.cpp:377-397).
//
//   1. 63-bit Morton keys of the FP64 positions in the global bounding box;
//      CUB radix sort; particles permuted into key order.
//   2. Binary radix tree over the sorted keys (Karras 2012): internal nodes
//      0..n-2, leaf node n-1+p for particle p; one thread per internal node.
//   3. Bottom-up refit (second arrival at a node combines its children):
//      FP32 outward-rounded bounding box, max h, monopole in FP64 (mass,
//      centre of mass, mass-weighted eps^2 as GravityMonopole,
//      hdr_gravity.hpp:37-49).  Particle ranges come from the tree build.
//   4. i-groups ("walks"): maximal subtrees with <= n_group particles.
//   5. Lists: each group's region is first expanded breadth-first into
//      traversal tasks (subtrees), then one warp per task runs a
//      warp-cooperative batched-DFS traversal with a shared-memory stack,
//      once: it counts the task's entries and appends them, in traversal
//      order, to 128-entry chunks taken from a pool; after a scan of the
//      counts, copy_lists moves each task's chunks to its list offset, so
//      list order is deterministic:
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
    dbl4 *mom;        // centre of mass x, y, z; w = mass
    double *eps2;     // mass-weighted eps^2
    int *visit;       // refit arrival counters
    float4 *flo;      // FP32 traversal copies: lo (rounded down), w = max h (up)
    float4 *fhi;      // hi (rounded up), w = largest box side (up)
    float4 *fmom;     // centre of mass, mass
    float4 *ptest;    // per particle: position (nearest), h (rounded up)
    // quadrupole (when the system uses it, else null): traceless
    // Q = sum m (3 d d^T - |d|^2 I) about the centre of mass, FP64 as
    // (xx, yy, zz, xy, xz, yz) per node, and its FP32 copy
    // fq0 = (xx, yy, zz, xy), fq1 = (xz, yz, 0, 0)
    double *quad;
    float4 *fq0, *fq1;
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
    // the scale once per block (an FP64 division per thread would dominate)
    __shared__ double s_scale;
    if (threadIdx.x == 0) {
        double span = fmax(fmax(box[3] - lx, box[4] - ly), box[5] - lz);
        span = span > 0.0 ? span : 1.0;
        s_scale = 2097151.0 / span;
    }
    __syncthreads();
    const double s = s_scale;
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

__device__ __forceinline__ void radix_node(const uint64_t *k, int n, Nodes t, int i) {
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
    t.first[i] = min(i, j);
    t.count[i] = abs(j - i) + 1;
    t.parent[left] = i;
    t.parent[right] = i;
    if (i == 0) t.parent[0] = -1;
}

// Internal node i covers the particle range between i and j (Karras's
// determineRange); its first particle and count are written here, the
// leaves' trivially.
__global__ void build_radix_tree(const uint64_t *k, int n, Nodes t) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        t.first[n - 1 + p] = p;
        t.count[n - 1 + p] = 1;
        if (n == 1) t.parent[0] = -1;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x)
        radix_node(k, n, t, i);
}

// ---- 3. refit ----------------------------------------------------------------
// Refit data of a node.  The traversal uses FP32 boxes rounded outwards
// (flo.w = max h rounded up; fhi.w = largest box side, filled at store
// time), so the boxes are merged in FP32 (min/max of conservative boxes stays
// conservative) and no FP64 box is kept.  The monopole is accumulated in FP64
// as unnormalised sums: sm = (sum m x, sum m y, sum m z, sum m), se = sum m eps^2.
struct NodeData {
    dbl4 sm;
    float4 flo, fhi;
    double se;
};

__device__ __forceinline__ NodeData combine(const NodeData &a, const NodeData &b) {
    NodeData r;
    r.sm = make_dbl4(a.sm.x + b.sm.x, a.sm.y + b.sm.y, a.sm.z + b.sm.z, a.sm.w + b.sm.w);
    r.se = a.se + b.se;
    r.flo = make_float4(fminf(a.flo.x, b.flo.x), fminf(a.flo.y, b.flo.y), fminf(a.flo.z, b.flo.z),
                        fmaxf(a.flo.w, b.flo.w));
    r.fhi = make_float4(fmaxf(a.fhi.x, b.fhi.x), fmaxf(a.fhi.y, b.fhi.y), fmaxf(a.fhi.z, b.fhi.z), 0.0f);
    return r;
}

__device__ __forceinline__ NodeData leaf_data(const dbl4 &x, double h, double eps2) {
    NodeData d;
    d.sm = make_dbl4(x.w * x.x, x.w * x.y, x.w * x.z, x.w);
    d.se = x.w * eps2;
    d.flo = make_float4(__double2float_rd(x.x), __double2float_rd(x.y), __double2float_rd(x.z),
                        __double2float_ru(h));
    d.fhi = make_float4(__double2float_ru(x.x), __double2float_ru(x.y), __double2float_ru(x.z), 0.0f);
    return d;
}

// Writes an internal node during the climb: FP32 boxes with the side length
// (rounded up) and the monopole still as unnormalised sums (sum m x, sum m;
// sum m eps^2), so that no division sits on the climb's critical path;
// normalise_nodes turns them into centre of mass and mean eps^2 afterwards.
__device__ __forceinline__ void store_node(const Nodes &t, int node, const NodeData &d) {
    const float size = fmaxf(fmaxf(__fsub_ru(d.fhi.x, d.flo.x), __fsub_ru(d.fhi.y, d.flo.y)),
                             __fsub_ru(d.fhi.z, d.flo.z));
    t.flo[node] = d.flo;
    t.fhi[node] = make_float4(d.fhi.x, d.fhi.y, d.fhi.z, size);
    t.mom[node] = d.sm;
    t.eps2[node] = d.se;
}

// A node written by another SM, back as refit data (L1 bypassed): leaves
// hold (x, m) and eps^2, internal nodes the sums of the climb.
__device__ __forceinline__ NodeData load_node_cg(const Nodes &t, int node, int n) {
    NodeData d;
    const double2 *q = reinterpret_cast<const double2 *>(&t.mom[node]);
    const double2 a = __ldcg(q), b = __ldcg(q + 1);
    if (node >= n - 1) {
        d.sm = make_dbl4(b.y * a.x, b.y * a.y, b.y * b.x, b.y);
        d.se = b.y * __ldcg(&t.eps2[node]);
    } else {
        d.sm = make_dbl4(a.x, a.y, b.x, b.y);
        d.se = __ldcg(&t.eps2[node]);
    }
    d.flo = __ldcg(&t.flo[node]);
    d.fhi = __ldcg(&t.fhi[node]);
    return d;
}

// Quadrupole runs accumulate second moments about the step's bounding-box
// centre o during the climb, S = sum m (x - o)(x - o)^T (plain sums, no
// division), in t.quad; normalise_nodes turns them into the traceless
// quadrupole about the node's centre of mass c, Q = 3 C - tr(C) I with
// C = S - m d d^T, d = c - o (FP64: the cancellation of S against m d d^T
// costs ~1e-9 relative at the box sizes and node sizes of a collision).
// Leaves end with Q = 0.
struct Quad {
    double q[6];   // xx, yy, zz, xy, xz, yz
};

__device__ __forceinline__ double3 box_centre(const double *box) {
    return make_double3(0.5 * (box[0] + box[3]), 0.5 * (box[1] + box[4]), 0.5 * (box[2] + box[5]));
}

__device__ __forceinline__ Quad leaf_moments(const dbl4 &x, const double3 &o) {
    const double dx = x.x - o.x, dy = x.y - o.y, dz = x.z - o.z, m = x.w;
    Quad q;
    q.q[0] = m * dx * dx; q.q[1] = m * dy * dy; q.q[2] = m * dz * dz;
    q.q[3] = m * dx * dy; q.q[4] = m * dx * dz; q.q[5] = m * dy * dz;
    return q;
}

__device__ __forceinline__ Quad add_moments(const Quad &a, const Quad &b) {
    Quad r;
    for (int k = 0; k < 6; ++k) r.q[k] = a.q[k] + b.q[k];
    return r;
}

__device__ __forceinline__ void store_moments(const Nodes &t, int node, const Quad &q) {
    for (int k = 0; k < 6; ++k) t.quad[6 * (size_t)node + k] = q.q[k];
}

__device__ __forceinline__ void store_quad(const Nodes &t, int node, const Quad &q) {
    store_moments(t, node, q);
    t.fq0[node] = make_float4((float)q.q[0], (float)q.q[1], (float)q.q[2], (float)q.q[3]);
    t.fq1[node] = make_float4((float)q.q[4], (float)q.q[5], 0.0f, 0.0f);
}

// Second moments of a node written by another SM: a leaf's from its particle
// (the leaf itself stores Q = 0), an internal node's from the climb.
__device__ __forceinline__ Quad load_moments_cg(const Nodes &t, int node, int n, const double3 &o) {
    if (node >= n - 1) {
        const double2 *p = reinterpret_cast<const double2 *>(&t.mom[node]);
        const double2 a = __ldcg(p), b = __ldcg(p + 1);
        return leaf_moments(make_dbl4(a.x, a.y, b.x, b.y), o);
    }
    Quad q;
    for (int k = 0; k < 6; ++k) q.q[k] = __ldcg(&t.quad[6 * (size_t)node + k]);
    return q;
}

// Centre of mass, mass-weighted eps^2, the quadrupole (quadrupole runs) and
// the FP32 copy of the internal nodes from their sums (leaves hold the
// particle's own values).
__global__ void normalise_nodes(int n, Nodes t, const double *box, bool quad) {
    const double3 o = quad ? box_centre(box) : make_double3(0.0, 0.0, 0.0);
    for (int node = blockIdx.x * blockDim.x + threadIdx.x; node < n - 1; node += gridDim.x * blockDim.x) {
        const dbl4 s = t.mom[node];
        dbl4 m;
        double e2;
        if (s.w > 0.0) {
            const double mi = 1.0 / s.w;
            m = make_dbl4(s.x * mi, s.y * mi, s.z * mi, s.w);
            e2 = t.eps2[node] * mi;
        } else {
            const float4 lo = t.flo[node], hi = t.fhi[node];
            m = make_dbl4(0.5 * ((double)lo.x + hi.x), 0.5 * ((double)lo.y + hi.y), 0.5 * ((double)lo.z + hi.z),
                          0.0);
            e2 = 0.0;
        }
        t.mom[node] = m;
        t.eps2[node] = e2;
        t.fmom[node] = make_float4((float)m.x, (float)m.y, (float)m.z, (float)m.w);
        if (quad) {
            Quad q;
            for (int k = 0; k < 6; ++k) q.q[k] = 0.0;
            if (s.w > 0.0) {
                const double dx = m.x - o.x, dy = m.y - o.y, dz = m.z - o.z;
                const double *S = t.quad + 6 * (size_t)node;
                const double cxx = S[0] - s.w * dx * dx, cyy = S[1] - s.w * dy * dy, czz = S[2] - s.w * dz * dz;
                const double tr = cxx + cyy + czz;
                q.q[0] = 3.0 * cxx - tr;
                q.q[1] = 3.0 * cyy - tr;
                q.q[2] = 3.0 * czz - tr;
                q.q[3] = 3.0 * (S[3] - s.w * dx * dy);
                q.q[4] = 3.0 * (S[4] - s.w * dx * dz);
                q.q[5] = 3.0 * (S[5] - s.w * dy * dz);
            }
            store_quad(t, node, q);
        }
    }
}

// The refit runs in two parts.  Bottom: every maximal subtree of at most
// REFIT_B particles is refitted by one block in shared memory (one thread per
// leaf climbing while it is the second arrival at a node, block-scope
// counters).  Top: one thread per such subtree climbs the few nodes above
// them with device-scope arrival counters.  Threads therefore never hold a
// warp for a climb through the whole tree.
constexpr int REFIT_B = 128;

// Roots of the bottom subtrees: count <= REFIT_B, parent's count > REFIT_B.
__global__ void mark_subtrees(Nodes t, int n, int *roots, int *n_roots) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < 2 * n - 1; v += gridDim.x * blockDim.x) {
        const int p = t.parent[v];
        if (t.count[v] <= REFIT_B && (p < 0 || t.count[p] > REFIT_B)) roots[atomicAdd(n_roots, 1)] = v;
    }
}

template <bool QUAD>
__global__ void __launch_bounds__(REFIT_B)
refit_bottom(const dbl4 *pos, const double *h, const double *eps2, int n, Nodes t, const int *roots,
             const int *n_roots, const double *box) {
    // slots 0..B-1: internal node (index - first), B..2B-1: leaf (particle - first)
    __shared__ NodeData sd[2 * REFIT_B];
    __shared__ Quad sq[QUAD ? 2 * REFIT_B : 1];
    __shared__ int visit[REFIT_B];
    const int nr = *n_roots;
    const double3 o = QUAD ? box_centre(box) : make_double3(0.0, 0.0, 0.0);
    for (int r = blockIdx.x; r < nr; r += gridDim.x) {
        const int root = roots[r];
        const int a = t.first[root];
        const int c = t.count[root];
        if (c < 1 || c > REFIT_B) continue;   // not a bottom subtree (block-uniform)
        visit[threadIdx.x] = 0;
        __syncthreads();
        if ((int)threadIdx.x < c) {
            const int p = a + threadIdx.x;
            const dbl4 x = pos[p];
            const double hp = h[p], ep = eps2[p];
            NodeData d = leaf_data(x, hp, ep);
            int node = n - 1 + p;
            // leaf: exact position, mass and eps^2
            t.flo[node] = d.flo;
            t.fhi[node] = make_float4(d.fhi.x, d.fhi.y, d.fhi.z,
                                      fmaxf(fmaxf(__fsub_ru(d.fhi.x, d.flo.x), __fsub_ru(d.fhi.y, d.flo.y)),
                                            __fsub_ru(d.fhi.z, d.flo.z)));
            t.mom[node] = x;
            t.eps2[node] = ep;
            t.fmom[node] = make_float4((float)x.x, (float)x.y, (float)x.z, (float)x.w);
            t.ptest[p] = make_float4((float)x.x, (float)x.y, (float)x.z, __double2float_ru(hp));
            sd[REFIT_B + threadIdx.x] = d;
            // a leaf's stored quadrupole is 0, written once when the
            // buffers are allocated; only its second moments enter the climb
            if (QUAD) sq[REFIT_B + threadIdx.x] = leaf_moments(x, o);
            while (node != root) {
                node = t.parent[node];
                // internal nodes of the subtree have indices in [a, a + c)
                if (node < a || node >= a + c) break;
                __threadfence_block();
                if (atomicAdd(&visit[node - a], 1) == 0) break;   // sibling not finished yet
                __threadfence_block();
                const int2 ch = t.child[node];
                const int sa = (ch.x >= n - 1) ? REFIT_B + (ch.x - (n - 1) - a) : ch.x - a;
                const int sb = (ch.y >= n - 1) ? REFIT_B + (ch.y - (n - 1) - a) : ch.y - a;
                if (sa < 0 || sa >= 2 * REFIT_B || sb < 0 || sb >= 2 * REFIT_B) break;
                if (QUAD) {
                    const Quad q = add_moments(sq[sa], sq[sb]);
                    sq[node - a] = q;
                    store_moments(t, node, q);
                }
                d = combine(sd[sa], sd[sb]);
                sd[node - a] = d;
                store_node(t, node, d);
            }
        }
        __syncthreads();
    }
}

// visit[] (internal nodes) is zero on entry.
template <bool QUAD>
__global__ void refit_top(int n, Nodes t, const int *roots, const int *n_roots, const double *box) {
    const int nr = *n_roots;
    const double3 o = QUAD ? box_centre(box) : make_double3(0.0, 0.0, 0.0);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nr; r += gridDim.x * blockDim.x) {
        int node = t.parent[roots[r]];
        while (node >= 0) {
            // acq_rel arrival: the first arriver's node writes are released by
            // its atomic, the second arriver acquires them with its own
            int arrived;
            asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;"
                         : "=r"(arrived) : "l"(&t.visit[node]) : "memory");
            if (arrived == 0) break;   // sibling not finished yet
            const int2 ch = t.child[node];
            const NodeData da = load_node_cg(t, ch.x, n), db = load_node_cg(t, ch.y, n);
            if (QUAD) store_moments(t, node, add_moments(load_moments_cg(t, ch.x, n, o), load_moments_cg(t, ch.y, n, o)));
            store_node(t, node, combine(da, db));
            node = t.parent[node];
        }
    }
}

// Refit after a change of h alone (positions, masses, boxes, centres of mass
// and quadrupoles unchanged): only the largest h of each node (flo.w, and a
// particle's ptest.w) and its sum m eps^2 are recomputed, with the same
// operations in the same order as the full refit, so the node data are bit
// for bit those of a full refit.  Single-field stores leave the rest of each
// record untouched.
__global__ void __launch_bounds__(REFIT_B)
refit_bottom_h(const double *h, const double *eps2, int n, Nodes t, const int *roots, const int *n_roots) {
    __shared__ float sh[2 * REFIT_B];    // largest h (rounded up), slots as refit_bottom
    __shared__ double se[2 * REFIT_B];   // sum m eps^2
    __shared__ int visit[REFIT_B];
    const int nr = *n_roots;
    for (int r = blockIdx.x; r < nr; r += gridDim.x) {
        const int root = roots[r];
        const int a = t.first[root];
        const int c = t.count[root];
        if (c < 1 || c > REFIT_B) continue;   // not a bottom subtree (block-uniform)
        visit[threadIdx.x] = 0;
        __syncthreads();
        if ((int)threadIdx.x < c) {
            const int p = a + threadIdx.x;
            int node = n - 1 + p;
            const double hp = h[p], ep = eps2[p];
            const double m = t.mom[node].w;   // a leaf holds its particle's (x, m)
            float hw = __double2float_ru(hp);
            double s = m * ep;
            t.flo[node].w = hw;
            t.eps2[node] = ep;
            t.ptest[p].w = hw;
            sh[REFIT_B + threadIdx.x] = hw;
            se[REFIT_B + threadIdx.x] = s;
            while (node != root) {
                node = t.parent[node];
                if (node < a || node >= a + c) break;
                __threadfence_block();
                if (atomicAdd(&visit[node - a], 1) == 0) break;   // sibling not finished yet
                __threadfence_block();
                const int2 ch = t.child[node];
                const int sa = (ch.x >= n - 1) ? REFIT_B + (ch.x - (n - 1) - a) : ch.x - a;
                const int sb = (ch.y >= n - 1) ? REFIT_B + (ch.y - (n - 1) - a) : ch.y - a;
                if (sa < 0 || sa >= 2 * REFIT_B || sb < 0 || sb >= 2 * REFIT_B) break;
                hw = fmaxf(sh[sa], sh[sb]);
                s = se[sa] + se[sb];
                sh[node - a] = hw;
                se[node - a] = s;
                t.flo[node].w = hw;
                t.eps2[node] = s;
            }
        }
        __syncthreads();
    }
}

// visit[] (internal nodes) is zero on entry.
__global__ void refit_top_h(int n, Nodes t, const int *roots, const int *n_roots) {
    const int nr = *n_roots;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nr; r += gridDim.x * blockDim.x) {
        int node = t.parent[roots[r]];
        while (node >= 0) {
            int arrived;
            asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;"
                         : "=r"(arrived) : "l"(&t.visit[node]) : "memory");
            if (arrived == 0) break;   // sibling not finished yet
            const int2 ch = t.child[node];
            const int cs[2] = {ch.x, ch.y};
            float hw[2];
            double s[2];
            for (int k = 0; k < 2; ++k) {
                const int v = cs[k];
                hw[k] = __ldcg(&t.flo[v].w);
                // a leaf stores its particle's eps^2, an internal node the sum
                s[k] = (v >= n - 1) ? __ldcg(&t.mom[v].w) * __ldcg(&t.eps2[v]) : __ldcg(&t.eps2[v]);
            }
            t.flo[node].w = fmaxf(hw[0], hw[1]);
            t.eps2[node] = s[0] + s[1];
            node = t.parent[node];
        }
    }
}

// Mass-weighted mean eps^2 of the internal nodes after refit_*_h (their
// centres of mass and masses are already normalised).
__global__ void normalise_eps2(int n, Nodes t) {
    for (int node = blockIdx.x * blockDim.x + threadIdx.x; node < n - 1; node += gridDim.x * blockDim.x) {
        const double m = t.mom[node].w;
        t.eps2[node] = (m > 0.0) ? t.eps2[node] * (1.0 / m) : 0.0;
    }
}

// ---- 4. groups -------------------------------------------------------------
// flag[first particle of a group root] = 1, root_at[first] = node.
__global__ void mark_groups(Nodes t, int n, int n_group, int *flag, int *root_at) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < 2 * n - 1; v += gridDim.x * blockDim.x) {
        const int c = t.count[v];
        const int p = t.parent[v];
        const int pc = (p >= 0) ? t.count[p] : 0x7fffffff;
        if (c <= n_group && pc > n_group) {
            const int f = t.first[v];
            flag[f] = 1;
            root_at[f] = v;
        }
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
    // traversal tasks: (group, start node); see list_tasks
    const int2 *tasks;
    const int *n_tasks;     // device count of tasks
    // pass 1 writes counts per task, pass 2 fills at offsets
    int *count_out;
    const int *offset;      // exclusive scan of the task counts (fill pass)
    int *j_idx;
    long long capacity;     // entries available in j_idx
    int *error;             // bit 1: stack overflow, bit 2: capacity exceeded
    // chunk pass: each task appends its entries to LIST_CHUNK-entry chunks
    // taken from a pool (pool_next counts the chunks handed out); chain
    // holds the chunk ids of task t at [t * chain_max, ...).  pool_error:
    // bit 1 pool exhausted, bit 2 a task needed more than chain_max chunks
    int *pool;
    long long pool_chunks;
    int *pool_next;
    int *chain;
    int chain_max;
    int *pool_error;
    int *task_queue;        // next task to traverse (0 at launch): warps take tasks as they finish
};

constexpr int LIST_CHUNK = 128;   // entries per pool chunk (a multiple of 32)
enum { PASS_COUNT = 0, PASS_FILL = 1, PASS_CHUNK = 2 };

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

// Region of group g for the node and particle tests: box (FP32, outward
// rounded) and radius.
__device__ __forceinline__ float group_radius(const ListArgs &a, int mode, int g, const float4 &glo) {
    if (mode == GATHER) return __double2float_ru(a.r_group[g]);
    if (mode == SYMMETRIC) return glo.w;   // max h of the group (rounded up)
    return 0.0f;
}

// Node test of the traversal: 0 = reject, 1 = bucket (test its particles),
// 2 = open (descend), 3 = accept as a monopole (gravity).
template <int MODE>
__device__ __forceinline__ int node_class(const ListArgs &a, int node, const float4 &glo, const float4 &ghi,
                                          float rg, float slack) {
    const float4 lo = a.t.flo[node];
    const float4 hi = a.t.fhi[node];
    const bool leafish = (node >= a.n - 1) || a.t.count[node] <= a.n_leaf;
    if (MODE == GRAVITY) {
        const float4 m = a.t.fmom[node];
        const float d2 = point_box_d2f(m.x, m.y, m.z, glo, ghi);
        if (d2 > hi.w * hi.w * a.inv_theta2) return 3;
        return leafish ? 1 : 2;
    }
    const float r = widen(MODE == SYMMETRIC ? fmaxf(rg, lo.w) : rg, slack);
    if (box_box_d2f(glo, ghi, lo, hi) > r * r) return 0;
    return leafish ? 1 : 2;
}

__device__ __forceinline__ float coord_slack(const double *box) {
    // coordinates were rounded to FP32: |error| <= 2^-24 max|x| per axis
    const double cmax = fmax(fmax(fmax(fabs(box[0]), fabs(box[3])), fmax(fabs(box[1]), fabs(box[4]))),
                             fmax(fabs(box[2]), fabs(box[5])));
    return (float)(4.0e-7 * cmax);
}

// Traversal tasks.  One warp per group expands the nodes its region reaches
// breadth-first, opening only nodes of more than TASK_SPLIT particles, up to
// TASK_CAP nodes; each remaining node becomes a task (group, start node) that
// one warp traverses depth-first.  A group whose region covers many
// particles is thereby spread over many warps instead of one long traversal,
// and the order of its list (tasks in frontier order, each in depth-first
// order) stays deterministic.  WRITE = false counts tasks per group,
// WRITE = true writes them at the scanned offsets.
constexpr int TASK_CAP = 64;
constexpr int TASK_SPLIT = 2048;

template <int MODE, bool WRITE>
__global__ void __launch_bounds__(TRAV_WARPS * 32)
list_tasks(ListArgs a, int *task_count, const int *task_off, int2 *tasks, int task_cap) {
    __shared__ int fr[TRAV_WARPS][2][TASK_CAP];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int n_groups = *a.n_groups;
    const int warps = gridDim.x * TRAV_WARPS;
    const float slack = coord_slack(a.box);
    for (int g = blockIdx.x * TRAV_WARPS + wid; g < n_groups; g += warps) {
        const int gn = a.group_node[g];
        const float4 glo = a.t.flo[gn];
        const float4 ghi = a.t.fhi[gn];
        const float rg = group_radius(a, MODE, g, glo);
        int cur = 0, nf = 1;
        if (lane == 0) fr[wid][0][0] = a.root;
        __syncwarp();
        for (;;) {
            // classify the frontier (two nodes per lane)
            int nd[2], cls[2], split[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int k = lane + 32 * u;
                nd[u] = (k < nf) ? fr[wid][cur][k] : -1;
                cls[u] = 0;
                split[u] = 0;
                if (nd[u] >= 0) {
                    cls[u] = node_class<MODE>(a, nd[u], glo, ghi, rg, slack);
                    // gravity lists are of uniform length: one task per group
                    split[u] = (MODE != GRAVITY && cls[u] == 2 && a.t.count[nd[u]] > TASK_SPLIT) ? 1 : 0;
                }
            }
            // size of the next frontier: split nodes give two, kept nodes one
            int w0 = (cls[0] == 0) ? 0 : 1 + split[0];
            int w1 = (cls[1] == 0) ? 0 : 1 + split[1];
            int inc = w0 + w1;
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(FULL, inc, o);
                if (lane >= o) inc += v;
            }
            const int next = __shfl_sync(FULL, inc, 31);
            const bool any_split = __any_sync(FULL, split[0] | split[1]);
            const bool expand = any_split && next <= TASK_CAP;
            if (!expand) {
                // final frontier: the nodes not rejected, in order
                const unsigned m0 = __ballot_sync(FULL, cls[0] != 0);
                const unsigned m1 = __ballot_sync(FULL, cls[1] != 0);
                const int c0 = __popc(m0);
                if (WRITE) {
                    const long long base = task_off[g];
                    if (cls[0] != 0) {
                        const long long w = base + __popc(m0 & lt_mask);
                        if (w < task_cap) tasks[w] = make_int2(g, nd[0]);
                        else atomicOr(a.error, 2);
                    }
                    if (cls[1] != 0) {
                        const long long w = base + c0 + __popc(m1 & lt_mask);
                        if (w < task_cap) tasks[w] = make_int2(g, nd[1]);
                        else atomicOr(a.error, 2);
                    }
                } else if (lane == 0) {
                    task_count[g] = c0 + __popc(m1);
                }
                break;
            }
            const int nxt = cur ^ 1;
            int pos = inc - w0 - w1;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (cls[u] != 0) {
                    if (split[u]) {
                        const int2 c = a.t.child[nd[u]];
                        fr[wid][nxt][pos] = c.x;
                        fr[wid][nxt][pos + 1] = c.y;
                        pos += 2;
                    } else {
                        fr[wid][nxt][pos] = nd[u];
                        pos += 1;
                    }
                }
            }
            cur = nxt;
            nf = next;
            __syncwarp();
        }
        __syncwarp();
    }
}

// Groups' list offsets and lengths from their tasks' (each group's tasks are
// consecutive): off[g] = task_loff[task_off[g]], cnt[g] = its entries.
// Entries g in [n_groups, n] get the total and 0.
// Task offsets beyond the task capacity (an overflow already flagged as an
// error) are clamped to it.
__global__ void group_lists(int n, const int *n_groups, const int *task_off, const int *task_loff, int task_cap,
                            int *off, int *cnt) {
    const int ng = *n_groups;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g <= n; g += gridDim.x * blockDim.x) {
        const int gg = g < ng ? g : ng;
        const int o = task_loff[min(task_off[gg], task_cap)];
        off[g] = o;
        cnt[g] = (g < ng) ? task_loff[min(task_off[g + 1], task_cap)] - o : 0;
    }
}

// One traversal per task (one warp each).  PASS_COUNT counts the entries of
// every task; PASS_FILL writes them at the scanned task offsets; PASS_CHUNK
// counts them and writes them, in the same order, into pool chunks, which
// copy_lists moves to the scanned offsets (one traversal instead of two).
template <int MODE, int PASS>
__global__ void __launch_bounds__(TRAV_WARPS * 32) build_lists(ListArgs a) {
    constexpr bool FILL = PASS == PASS_FILL;
    __shared__ int stack[TRAV_WARPS][STACK];
    __shared__ int cand[TRAV_WARPS][CAND];
    __shared__ int cpre[TRAV_WARPS][CAND + 1];
    __shared__ int pidx[TRAV_WARPS][CAND * MAX_LEAF];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int n_tasks = *a.n_tasks;
    const float slack = coord_slack(a.box);
    // tasks differ in length: each warp takes the next one when it is done
    // (the lists do not depend on the order, each task writing its own chunks)
    auto next_task = [&]() {
        int t = 0;
        if (lane == 0) t = atomicAdd(a.task_queue, 1);
        return __shfl_sync(FULL, t, 0);
    };
    for (int task = next_task(); task < n_tasks; task = next_task()) {
        const int2 tk = a.tasks[task];
        const int g = tk.x;
        const int gn = a.group_node[g];
        const float4 glo = a.t.flo[gn];
        const float4 ghi = a.t.fhi[gn];
        const float rg = group_radius(a, MODE, g, glo);
        long long out = FILL ? (long long)a.offset[task] : 0;
        int total = 0;
        // chunk pass: current chunk, its fill, chunks taken by this task
        int cchunk = -1, cfill = LIST_CHUNK, nch = 0;
        bool pool_bad = false;
        // appends the lanes' accepted entries (ballot order) to the task's chunks
        auto emit = [&](bool ok, int value) {
            const unsigned m = __ballot_sync(FULL, ok);
            if (m == 0u) return;
            const int cnt = __popc(m);
            int nchunk = -1;
            if (cfill + cnt > LIST_CHUNK) {
                if (lane == 0) nchunk = atomicAdd(a.pool_next, 1);
                nchunk = __shfl_sync(FULL, nchunk, 0);
                if (nchunk >= a.pool_chunks || nch >= a.chain_max) {
                    if (lane == 0) atomicOr(a.pool_error, nchunk >= a.pool_chunks ? 1 : 2);
                    pool_bad = true;
                } else if (lane == 0) {
                    a.chain[(size_t)task * a.chain_max + nch] = nchunk;
                }
                ++nch;
            }
            if (ok && !pool_bad) {
                const int pos = cfill + __popc(m & lt_mask);
                const int ch = pos < LIST_CHUNK ? cchunk : nchunk;
                a.pool[(size_t)ch * LIST_CHUNK + (pos < LIST_CHUNK ? pos : pos - LIST_CHUNK)] = value;
            }
            if (nchunk >= 0) {
                cchunk = nchunk;
                cfill = cfill + cnt - LIST_CHUNK;
            } else {
                cfill += cnt;
            }
        };
        int sp = 1, nc = 0;
        if (lane == 0) stack[wid][0] = tk.y;
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
                    const int c = node_class<MODE>(a, node, glo, ghi, rg, slack);
                    accept = c == 3;
                    bucket = c == 1;
                    push = c == 2;
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
                    if (PASS == PASS_CHUNK) emit(accept, a.n + node);
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
                // four 32-particle batches per round: their loads are issued
                // together, the accepted particles keep the batch order
                for (int b = 0; b < tot; b += 128) {
                    int p[4];
                    float4 x[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int k = b + 32 * u + lane;
                        p[u] = (k < tot) ? pidx[wid][k] : -1;
                    }
                    if (MODE != GRAVITY) {
#pragma unroll
                        for (int u = 0; u < 4; ++u)
                            if (p[u] >= 0) x[u] = a.t.ptest[p[u]];
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        bool ok = p[u] >= 0;
                        if (ok && MODE != GRAVITY) {
                            const float r = widen(MODE == SYMMETRIC ? fmaxf(rg, x[u].w) : rg, slack);
                            ok = point_box_d2f(x[u].x, x[u].y, x[u].z, glo, ghi) <= r * r;
                        }
                        if (PASS == PASS_CHUNK) emit(ok, p[u]);
                        const unsigned om = __ballot_sync(FULL, ok);
                        if (FILL && ok) {
                            const long long w = out + __popc(om & lt_mask);
                            if (w < a.capacity) a.j_idx[w] = p[u];
                            else atomicOr(a.error, 2);
                        }
                        out += __popc(om);
                        total += __popc(om);
                    }
                }
                nc = 0;
                __syncwarp();
            }
            if (overflow) break;
        }
        if (overflow && lane == 0) atomicOr(a.error, 1);
        if (!FILL && lane == 0) a.count_out[task] = total;
    }
}

// Moves each task's chunks (PASS_CHUNK) to its scanned list offset: one
// block per task, each thread copying every COPY_THREADS-th entry (all loads
// of a round in flight together; chunk ids come from L1 after the first
// thread).  After a pool or chain overflow nothing is copied and the
// list-capacity error is raised (the evaluation is then repeated with larger
// buffers).
constexpr int COPY_THREADS = 256;
__global__ void __launch_bounds__(COPY_THREADS) copy_lists(ListArgs a) {
    const int n_tasks = *a.n_tasks;
    if (*a.pool_error) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.error, 2);
        return;
    }
    for (int task = blockIdx.x; task < n_tasks; task += gridDim.x) {
        const int total = a.count_out[task];
        const long long off = a.offset[task];
        const int *chain = a.chain + (size_t)task * a.chain_max;
        for (int k = threadIdx.x; k < total; k += COPY_THREADS) {
            const int ch = chain[k / LIST_CHUNK];
            const long long w = off + k;
            if (w >= 0 && w < a.capacity) a.j_idx[w] = a.pool[(size_t)ch * LIST_CHUNK + (k % LIST_CHUNK)];
            else atomicOr(a.error, 2);
        }
    }
}

}  // namespace sphtree
