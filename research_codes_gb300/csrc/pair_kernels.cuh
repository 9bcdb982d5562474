// pair_kernels.cuh — the three SPH pair-interaction kernels.
//
// Design (shared by density, hydro and gravity):
//  * Work is a list of WorkItems (<= 32 i-particles of one walk).  A
//    persistent grid of warps pulls items from a global queue counter
//    (atomicAdd), so walks with very different neighbour counts balance across
//    the SMs.  Items may address their i-particles through an index list
//    (search-radius re-walks recompute only the particles still iterating).
//  * A warp streams its walk's j-list through a private 32-entry shared-memory
//    tile: lane k loads entry t+k (gathered through j_idx), converts it and
//    stores it; every lane then reads the tile by broadcast.  With n_i < 32
//    several lanes share one i-particle (tpi lanes, strided over the tile) and
//    are combined with warp shuffles.
//  * FP32C mode (F64 == false): the engine keeps double-float copies of the
//    particle state (hi = float(x), lo = float(x - hi)).  Staging forms
//    (hi_j - hi_c) + (lo_j - lo_c) relative to the item's first i-particle c
//    in FP32, so pair differences keep FP32 relative accuracy far from the
//    origin and across colliding streams, and no FP64 instruction runs in the
//    pair loops (GB300's FP64 rate is ~1/60 of FP32).  Each lane's per-tile
//    FP32 partial sums are folded into Kahan accumulators.
//  * FP64 mode (F64 == true): the same kernels in plain FP64 on global
//    coordinates without compensation: the "plain FP64 GPU" comparator.
#pragma once

#include "hydro_df.cuh"
#include "sph_device.cuh"

// Minimum resident blocks per SM requested from the compiler for the FP32C
// density, gravity and hydro kernels (register budget 65536 / (128 threads x
// blocks)).
#ifndef SPH_DENSITY_MIN_BLOCKS
#define SPH_DENSITY_MIN_BLOCKS 4
#endif
#ifndef SPH_GRAVITY_MIN_BLOCKS
#define SPH_GRAVITY_MIN_BLOCKS 4
#endif
// Unroll factors of the full-tile FP32C loops: f32x2 iterations (two entries
// each) of the gravity and packed density loops, entries of the hydro
// mark-only loop.
#ifndef SPH_GRAVITY_UNROLL
#define SPH_GRAVITY_UNROLL 16
#endif
#ifndef SPH_DENSITY_UNROLL
#define SPH_DENSITY_UNROLL 4
#endif
#ifndef SPH_HYDRO_MARK_UNROLL
#define SPH_HYDRO_MARK_UNROLL 16
#endif
// The double-float hydro pass (128 threads): 3 blocks per SM, 168 registers.
#ifndef SPH_HYDRO_DF_MIN_BLOCKS
#define SPH_HYDRO_DF_MIN_BLOCKS 3
#endif
#ifndef SPH_HYDRO_MIN_BLOCKS
#define SPH_HYDRO_MIN_BLOCKS 4
#endif

namespace sphk {

constexpr int GRAVITY_UNROLL = SPH_GRAVITY_UNROLL;
constexpr int DENSITY_UNROLL = SPH_DENSITY_UNROLL;
constexpr int HYDRO_MARK_UNROLL = SPH_HYDRO_MARK_UNROLL;

// Double-float particle records of FP32C mode.
struct F32Part {
    const float4 *phi;   // x_hi, y_hi, z_hi, mass
    const float4 *plo;   // x_lo, y_lo, z_lo, aux
    const float4 *vhi;   // vx_hi, vy_hi, vz_hi, aux
    const float4 *vlo;   // vx_lo, vy_lo, vz_lo, aux
};

__device__ __forceinline__ float df_diff(float hi, float lo, float chi, float clo) {
    return (hi - chi) + (lo - clo);
}

// Double-float split of an FP64 value: hi = float(x), lo = float(x - hi).
__device__ __forceinline__ float2 df_split(double x) {
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

struct ItemRef {   // decoded work item
    int walk, jb, nj, ni, tpi, sub, li, ii, ic;
    bool act;
};

__device__ __forceinline__ ItemRef decode(const WorkItem &it, const int *j_off, const int *i_list, int lane) {
    ItemRef r;
    r.walk = it.x;
    r.jb = j_off[it.x];
    r.nj = j_off[it.x + 1] - r.jb;
    r.ni = it.z;
    r.tpi = lanes_per_i(it.z);
    const int sh = ilog2_pow2(r.tpi);
    r.li = lane >> sh;
    r.sub = lane & (r.tpi - 1);
    r.act = r.li < it.z;
    const int k = it.y + (r.act ? r.li : 0);
    r.ii = i_list ? i_list[k] : k;
    r.ic = i_list ? i_list[it.y] : it.y;   // the item's centre particle
    return r;
}

// ---------------------------------------------------------------- density
struct DensityArgs {
    // FP64 records (i_pm is read in both modes for the i-particle's mass)
    const dbl4 *i_pm;       // x, y, z, mass
    const dbl4 *i_vel;      // vx, vy, vz, -
    const dbl4 *j_pm;
    const dbl4 *j_vel;
    // FP32C mode records (phi.w = mass)
    F32Part fi, fj;
    const long long *i_id;
    const long long *j_id;
    const double *i_ksr;    // first guess of h (DensityEPI::ksr)
    const double *i_rs;     // search radius (DensityEPI::rs)
    // work
    const WorkItem *items;
    int n_items;
    const int *n_items_dev; // when set, the item count is read from device memory
    const int *j_off;       // per walk: [j_off[w], j_off[w+1]) in j index space
    const int *j_idx;       // null: entries are j indices themselves
    const int *i_list;      // null: item i-particles are contiguous
    int *queue;             // item counter, 0 at launch
    // outputs, indexed like the i arrays
    double *o_dens, *o_divv, *o_rotv, *o_grdh, *o_ksr;
    long long *o_np;
    unsigned char *o_itr;
    double eta_ksrh;        // eta * ksrh
    double ksr_max;         // clamp of h (+inf disables)
    const double *ksr_max_dev;  // when set, the clamp is read from device memory
    // FP32C only: particles whose final h lies within amb_tol of rs (where
    // the search-radius decision h > rs of hdr_density.hpp:299 could come out
    // differently in FP64) are queued here for an FP64 recomputation
    int *amb_count;         // null disables the queue
    int *amb_i;             // queued particle index
    int *amb_w;             // its walk
    int amb_cap;
    float amb_tol;
    // Per-warp neighbour lists; null: every pass sweeps the walk's j-list.
    // Warp w of the grid (blockIdx.x * WARPS + warp) owns the int array
    // nbr[w * nbr_cap * 32, (w + 1) * nbr_cap * 32), entry c of lane l at
    // [c * 32 + l]; warps w >= nbr_warps sweep.  nbr_slack (> 1) is the list
    // radius in units of each i-particle's first-pass h.
    int *nbr = nullptr;
    int nbr_cap = 0;
    int nbr_warps = 0;
    float nbr_slack = 1.0f;
    // when set: pair evaluations performed, [0] the three density passes
    // ((j-entries kept by the support test x i-particles) of the swept passes
    // plus the list entries of the listed ones), [1] the gradient pass
    unsigned long long *n_eval = nullptr;
    // when set: [0] item passes (second, third, gradient) served from the
    // neighbour lists, [1] item passes that swept the walk's j-list
    unsigned long long *n_pass = nullptr;
};

template <bool B>
struct BTag {
    static constexpr bool value = B;
};

// The density functor of hdr_density.hpp:252-350 for one work item per warp:
// three fixed-point passes rho(h) -> h = eta ksrh (m / rho)^(1/3) from the
// first guess, then the gradient pass (grdh, divv, rotv) with the final h.
//
// Every pass can stream the walk's j-list through a shared ring (kept entries
// of each 32-entry chunk compacted by the item-box support test), which
// evaluates every kept entry for every i-particle of the item: ~10x more
// pairs than the kernel support holds.  With neighbour lists the first pass
// streams the list once with the support widened by nbr_slack and also writes,
// per lane, the j indices within nbr_slack * (first-pass h) of its
// i-particle; the second and third passes and the gradient pass then loop over
// each lane's own list (gathering the j records) whenever every h of the item
// has stayed within that radius and no lane's list overflowed nbr_cap;
// otherwise the pass sweeps.  Entries beyond a particle's support add exactly
// zero in both forms, so the two differ only in the grouping of the FP32
// partial sums.
template <bool F64, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, F64 ? 1 : SPH_DENSITY_MIN_BLOCKS)
density_kernel(const DensityArgs a) {
    typedef typename Real<F64>::T R;
    typedef typename Real<F64>::T4 R4;
    // per warp a 64-entry ring of compacted j records: entries accumulate
    // until 32 are ready, the pair loop consumes one 32-entry half at a time
    __shared__ R4 s_p[WARPS][64];
    __shared__ R4 s_v[WARPS][64];
    __shared__ float2 s_vl[WARPS][64];
    __shared__ long long s_id[WARPS][64];
    // FP32C density passes: the same ring as a structure of arrays, so that
    // two consecutive entries load as one f32x2 operand
    __shared__ __align__(16) float s_rx[F64 ? 1 : WARPS][64], s_ry[F64 ? 1 : WARPS][64],
        s_rz[F64 ? 1 : WARPS][64], s_rm[F64 ? 1 : WARPS][64];
    __shared__ int s_j[WARPS][64];   // j index of each ring entry (list-building pass)
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const unsigned lt = lanemask_lt();
    const int n_items = a.n_items_dev ? *a.n_items_dev : a.n_items;
    const double ksr_max = a.ksr_max_dev ? *a.ksr_max_dev : a.ksr_max;
    const int gw = blockIdx.x * WARPS + wid;
    // this lane's neighbour list: entry c at a.nbr[nlb + c * 32]
    const bool has_nl = a.nbr != nullptr && gw < a.nbr_warps;
    const int nlb = has_nl ? gw * a.nbr_cap * 32 + lane : 0;
    // list radius^2 over (first-pass h)^2, and the largest h (over the
    // first-pass h) a listed pass accepts: every pair with q < 1 then has r^2
    // below the list radius with a margin of 2e-5 over the rounding of both
    // tests
    const R nl_lim = (R)a.nbr_slack * (R)a.nbr_slack;
    const double nl_hmax = (double)a.nbr_slack * 0.99998;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.queue, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= n_items) return;
        const ItemRef r = decode(a.items[item], a.j_off, a.i_list, lane);
        const int tpi = r.tpi, sub = r.sub, ii = r.ii, nj = r.nj, jb = r.jb;

        // i-particle relative to the centre particle c (velocity, id, mass
        // and search radius are read where they are used, keeping the
        // registers of the passes free)
        R xi, yi, zi;
        float4 cph = make_float4(0, 0, 0, 0), cpl = cph;
        if (F64) {
            const dbl4 p = a.i_pm[ii];
            xi = (R)p.x; yi = (R)p.y; zi = (R)p.z;
        } else {
            cph = a.fi.phi[r.ic]; cpl = a.fi.plo[r.ic];
            const float4 ph = a.fi.phi[ii], pl = a.fi.plo[ii];
            xi = (R)df_diff(ph.x, pl.x, cph.x, cpl.x);
            yi = (R)df_diff(ph.y, pl.y, cph.y, cpl.y);
            zi = (R)df_diff(ph.z, pl.z, cph.z, cpl.z);
        }
        // The kernel is zero for r >= h, so a j-particle farther than the
        // largest h of the item from the item's box adds nothing to any sum
        // or count of this item: staging drops it before the pair loop.
        IBox<R> box;
        box.from_lanes(xi, yi, zi);
        double h = a.i_ksr[ii];
        // largest h a listed pass accepts for this lane
        const float nl_h = (float)(h * nl_hmax);
        R rho = 0;
        int np = 0;

        // One j record as loaded from memory (FP32C double-float or FP64).
        struct JRec {
            float4 ph, pl, vh, vl;
            dbl4 p, v;
            long long id;
        };
        auto jlist = [&](int k) -> int { return a.j_idx ? a.j_idx[jb + k] : jb + k; };
        auto load = [&](int j, bool with_v, JRec &q) {
            if constexpr (F64) {
                q.p = a.j_pm[j];
                if (with_v) q.v = a.j_vel[j];
            } else {
                q.ph = a.fj.phi[j];
                q.pl = a.fj.plo[j];
                if (with_v) {
                    q.vh = a.fj.vhi[j];
                    q.vl = a.fj.vlo[j];
                }
            }
            if (with_v) q.id = a.j_id[j];
        };
        // position of particle j in the frame of the pair loops (FP32C:
        // relative to the centre particle; FP64: absolute) and its mass
        auto jpos = [&](int j) -> R4 {
            if constexpr (F64) {
                const dbl4 p = a.j_pm[j];
                return Real<F64>::make4((R)p.x, (R)p.y, (R)p.z, (R)p.w);
            } else {
                const float4 ph = __ldg(&a.fj.phi[j]), pl = __ldg(&a.fj.plo[j]);
                return Real<F64>::make4(df_diff(ph.x, pl.x, cph.x, cpl.x), df_diff(ph.y, pl.y, cph.y, cpl.y),
                                        df_diff(ph.z, pl.z, cph.z, cpl.z), ph.w);
            }
        };
        // Streams the walk's list through the ring: lane k takes entry t+k,
        // entries that can lie within sqrt(rf2) of the item box are
        // compacted into the ring, and consume(base, n) runs whenever 32 are
        // ready (and once more for the rest).  Loads run one 32-entry chunk
        // ahead of their use (the list index two chunks ahead) so that their
        // latency overlaps the box test and the pair loops.  with_v also
        // stages velocities and ids (gradient pass), with_j the j indices.
        unsigned kept = 0;   // j-entries kept by the support test, all sweeps
        auto sweep = [&](const R rf2, const bool with_v, const bool with_j, auto &&consume) {
            int head = 0, fill = 0;
            JRec cur, nxt;
            int jn = 0, jnx = 0;
            if (lane < nj) {
                jnx = jlist(lane);
                load(jnx, with_v, nxt);
            }
            if (32 + lane < nj) jn = jlist(32 + lane);
            for (int t = 0; t < nj; t += 32) {
                cur = nxt;
                const int jc = jnx;
                const bool valid = t + lane < nj;
                if (t + 32 + lane < nj) {
                    jnx = jn;
                    load(jn, with_v, nxt);
                }
                if (t + 64 + lane < nj) jn = jlist(t + 64 + lane);
                bool keep = false;
                R4 p4;
                if (valid) {
                    if constexpr (F64) {
                        p4 = Real<F64>::make4((R)cur.p.x, (R)cur.p.y, (R)cur.p.z, (R)cur.p.w);
                    } else {
                        p4 = Real<F64>::make4((R)df_diff(cur.ph.x, cur.pl.x, cph.x, cpl.x),
                                              (R)df_diff(cur.ph.y, cur.pl.y, cph.y, cpl.y),
                                              (R)df_diff(cur.ph.z, cur.pl.z, cph.z, cpl.z), (R)cur.ph.w);
                    }
                    keep = !(box.d2(p4.x, p4.y, p4.z) > rf2);
                }
                const unsigned m = __ballot_sync(FULL, keep);
                if (keep) {
                    const int slot = (head + fill + __popc(m & lt)) & 63;
                    if (!F64 && !with_v) {
                        s_rx[wid][slot] = (float)p4.x;
                        s_ry[wid][slot] = (float)p4.y;
                        s_rz[wid][slot] = (float)p4.z;
                        s_rm[wid][slot] = (float)p4.w;
                    } else {
                        s_p[wid][slot] = p4;
                    }
                    if (with_v) {
                        if constexpr (F64) {
                            s_v[wid][slot] = Real<F64>::make4((R)cur.v.x, (R)cur.v.y, (R)cur.v.z, (R)0);
                        } else {
                            s_v[wid][slot] = Real<F64>::make4((R)cur.vh.x, (R)cur.vh.y, (R)cur.vh.z, (R)cur.vl.x);
                            s_vl[wid][slot] = make_float2(cur.vl.y, cur.vl.z);
                        }
                        s_id[wid][slot] = cur.id;
                    }
                    if (with_j) s_j[wid][slot] = jc;
                }
                fill += __popc(m);
                kept += __popc(m);
                __syncwarp();
                if (fill >= 32) {
                    consume(head, 32);
                    head ^= 32;
                    fill -= 32;
                }
            }
            if (fill > 0) consume(head, fill);
        };

        // neighbour list of this lane: its length (above nbr_cap the list is
        // unusable), appended by the first pass from the ring
        int ncnt = 0;
        bool nl_ok = false;
        unsigned ev_list = 0, ev_list_g = 0;   // list entries evaluated (this lane)
        int n_listed = 0;                      // of the 3 item passes after the first
        auto nl_push = [&](int head, unsigned msk) {
            while (msk) {
                const int k = __ffs(msk) - 1;
                msk &= msk - 1;
                if (ncnt < a.nbr_cap) a.nbr[nlb + ncnt * 32] = s_j[wid][head + k];
                ++ncnt;
            }
        };

        // three fixed-point passes, hdr_density.hpp:264-302
        for (int pass = 0; pass < 3; ++pass) {
            const R hinv = (R)1 / (R)h;
            const R hinv2 = hinv * hinv;
            const bool build = has_nl && pass == 0;
            const bool listed = pass > 0 && nl_ok && __all_sync(FULL, (float)h <= nl_h);
            Acc<F64> acc;
            int cnt = 0;
            R part = 0;
            // rho pair term m_j W0(q)/c0; neighbour count only in the last
            // pass (the only np the reference stores, :297)
            auto term = [&](const R4 pj, bool count) -> R {
                const R dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
                const R r2 = dx * dx + dy * dy + dz * dz;
                const R q = sqrt_q(r2, hinv2);
                const R u = max0((R)1 - q);
                const R u2 = u * u;
                if (count) cnt += (q < (R)1) ? 1 : 0;
                return pj.w * (u2 * u2 * ((R)1 + (R)4 * q));
            };
            // ring entry k; with mark set, bit k of *mark flags an entry
            // within the list radius
            auto pair = [&](int k, bool count, unsigned *mark) {
                R4 pj;
                if constexpr (F64) {
                    pj = s_p[wid][k];
                } else {
                    pj = Real<F64>::make4(s_rx[wid][k], s_ry[wid][k], s_rz[wid][k], s_rm[wid][k]);
                }
                part += term(pj, count);
                if (mark) {
                    const R dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
                    if ((dx * dx + dy * dy + dz * dz) * hinv2 < nl_lim) *mark |= 1u << (k & 31);
                }
            };
            // full FP32C tile: two entries per instruction (f32x2); even and
            // odd entries summed apart and combined at the end of the tile;
            // the list-building form also flags the entries within the list
            // radius
            auto run_packed = [&](int head, bool count, auto build_tag) {
                constexpr bool B = decltype(build_tag)::value;
                const f2 XI = f2_make((float)xi, (float)xi), YI = f2_make((float)yi, (float)yi);
                const f2 ZI = f2_make((float)zi, (float)zi), H2 = f2_make((float)hinv2, (float)hinv2);
                const f2 NEG = f2_make(-1.0f, -1.0f), ONE = f2_make(1.0f, 1.0f), FOUR = f2_make(4.0f, 4.0f);
                const float lim = (float)nl_lim;
                f2 PART = f2_make(0.0f, 0.0f);
                int c2 = 0;
                unsigned msk = 0;
#pragma unroll DENSITY_UNROLL
                for (int k = 0; k < 32; k += 2) {
                    const f2 DX = f2_fma(f2_lds(&s_rx[wid][head + k]), NEG, XI);
                    const f2 DY = f2_fma(f2_lds(&s_ry[wid][head + k]), NEG, YI);
                    const f2 DZ = f2_fma(f2_lds(&s_rz[wid][head + k]), NEG, ZI);
                    const float2 x2 = f2_get(f2_mul(f2_fma(DZ, DZ, f2_fma(DY, DY, f2_mul(DX, DX))), H2));
                    if constexpr (B) msk |= (x2.x < lim ? 1u << k : 0u) | (x2.y < lim ? 2u << k : 0u);
                    float q0, q1;
                    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(q0) : "f"(x2.x));
                    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(q1) : "f"(x2.y));
                    const f2 Q = f2_make(q0, q1);
                    const float2 u = f2_get(f2_fma(Q, NEG, ONE));
                    const f2 U = f2_make(max0(u.x), max0(u.y));
                    const f2 U2 = f2_mul(U, U);
                    PART = f2_fma(f2_lds(&s_rm[wid][head + k]), f2_mul(f2_mul(U2, U2), f2_fma(Q, FOUR, ONE)), PART);
                    if (count) c2 += (q0 < 1.0f ? 1 : 0) + (q1 < 1.0f ? 1 : 0);
                }
                const float2 ps = f2_get(PART);
                part = (R)(ps.x + ps.y);
                cnt += c2;
                if constexpr (B) nl_push(head, msk);
            };
            auto run = [&](int head, int n) {
                part = 0;
                if (!F64 && tpi == 1 && n == 32) {
                    if (build)
                        run_packed(head, false, BTag<true>());
                    else
                        run_packed(head, pass == 2, BTag<false>());
                } else {
                    unsigned msk = 0;
                    unsigned *mark = build ? &msk : nullptr;
                    if (tpi == 1 && n == 32) {
                        if (pass == 2) {
#pragma unroll 8
                            for (int k = 0; k < 32; ++k) pair(head + k, true, nullptr);
                        } else {
#pragma unroll 8
                            for (int k = 0; k < 32; ++k) pair(head + k, false, mark);
                        }
                    } else {
                        for (int k = sub; k < n; k += tpi) pair(head + k, pass == 2, mark);
                    }
                    if (build) nl_push(head, msk);
                }
                acc.add(part);
                __syncwarp();
            };
            if (listed) {
                // this lane's list, four entries per round (gathers first)
                const int cmax = (int)__reduce_max_sync(FULL, (unsigned)ncnt);
                for (int c0 = 0; c0 < cmax; c0 += 4) {
                    int jj[4];
                    R4 pj[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) jj[u] = (c0 + u < ncnt) ? a.nbr[nlb + (c0 + u) * 32] : -1;
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (jj[u] >= 0) pj[u] = jpos(jj[u]);
                    part = 0;
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (jj[u] >= 0) part += term(pj[u], pass == 2);
                    acc.add(part);
                }
                if (r.act) ev_list += (unsigned)ncnt;
                ++n_listed;
            } else {
                const R rf2 = support2<R>(build ? h * (double)a.nbr_slack : h);
                sweep(rf2, false, build, run);
            }
            if (build) nl_ok = __all_sync(FULL, ncnt <= a.nbr_cap);
            const double sum = seg_sum(acc.value(), tpi);
            const int c = (int)seg_sum((long long)cnt, tpi);
            const double mi = a.i_pm[ii].w;
            double hn;
            if (F64) {
                const double hinv_d = 1.0 / h;
                rho = (R)(CEFF0 * hinv_d * hinv_d * hinv_d * sum);
                hn = a.eta_ksrh * cbrt(mi / (double)rho);
            } else {
                // FP32 per-particle update (relative error ~1e-7, far inside
                // the 1e-5 budget) keeps the FP64 pipe out of the loop
                const float hinv_f = (float)hinv;
                const float rho_f = (float)CEFF0 * hinv_f * hinv_f * hinv_f * (float)sum;
                rho = (R)rho_f;
                hn = (double)((float)a.eta_ksrh * cbrtf((float)mi / rho_f));
            }
            hn = (hn < ksr_max) ? hn : ksr_max;
            np = c;
            h = hn;
        }
        // the search-radius decision of the last pass (hdr_density.hpp:299)
        const double rs_i = a.i_rs[ii];
        const bool itr = h > rs_i;
        if (!F64 && a.amb_count && r.act && sub == 0 && fabs(h - rs_i) <= (double)a.amb_tol * rs_i) {
            const int k = atomicAdd(a.amb_count, 1);
            if (k < a.amb_cap) {
                a.amb_i[k] = ii;
                a.amb_w[k] = r.walk;
            }
        }

        const unsigned kept_rho = kept;
        // gradient pass with the final h, hdr_density.hpp:304-349
        {
            const long long idi = a.i_id[ii];
            R vxi, vyi, vzi;
            float lxi = 0.0f, lyi = 0.0f, lzi = 0.0f;
            if (F64) {
                const dbl4 v = a.i_vel[ii];
                vxi = (R)v.x; vyi = (R)v.y; vzi = (R)v.z;
            } else {
                // velocities stay absolute hi/lo pairs and are differenced
                // per pair: an item may straddle two colliding streams
                const float4 vh = a.fi.vhi[ii], vl = a.fi.vlo[ii];
                vxi = vh.x; vyi = vh.y; vzi = vh.z;
                lxi = vl.x; lyi = vl.y; lzi = vl.z;
            }
            const R hinv = (R)1 / (R)h;
            Acc<F64> g_acc, d_acc, rx_acc, ry_acc, rz_acc;
            R pg = 0, pd = 0, prx = 0, pry = 0, prz = 0;
            // pair terms; (vx, vy, vz) the j velocity (FP32C: hi parts, with
            // the lo parts (lx, ly, lz) differenced apart)
            auto gpair = [&](const R4 pj, R vx, R vy, R vz, float lx, float ly, float lz, long long idj) {
                const R dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
                R ux = vxi - vx, uy = vyi - vy, uz = vzi - vz;
                if (!F64) {
                    ux += (R)(lxi - lx);
                    uy += (R)(lyi - ly);
                    uz += (R)(lzi - lz);
                }
                const R r2 = dx * dx + dy * dy + dz * dz;
                const R ri = (idi != idj) ? rsqrt_r(r2) : (R)0;
                const R q = r2 * ri * hinv;
                const R u = max0((R)1 - q);
                const R u2 = u * u;
                const R u3 = u2 * u;
                const R p14 = (R)1 + (R)4 * q;
                const R w0 = u2 * u2 * p14;            // W0 / c0
                const R w1 = w1_term(q, u, u2, u3, p14);   // W1 / c1
                pg += pj.w * ((R)(3.0 * CEFF0) * w0 + (R)CEFF1 * q * w1);
                const R dw = pj.w * w1 * ri;
                pd += (ux * dx + uy * dy + uz * dz) * dw;
                prx += (uy * dz - uz * dy) * dw;
                pry += (uz * dx - ux * dz) * dw;
                prz += (ux * dy - uy * dx) * dw;
            };
            auto pair = [&](int k) {
                const R4 vj = s_v[wid][k];
                const float2 vl = s_vl[wid][k];
                gpair(s_p[wid][k], vj.x, vj.y, vj.z, (float)vj.w, vl.x, vl.y, s_id[wid][k]);
            };
            auto fold = [&]() {
                g_acc.add(pg);
                d_acc.add(pd);
                rx_acc.add(prx);
                ry_acc.add(pry);
                rz_acc.add(prz);
                pg = 0; pd = 0; prx = 0; pry = 0; prz = 0;
            };
            // Each lane first marks the tile entries inside its own support
            // (r^2/h^2 below 1 + 2e-5, so every pair with q < 1 is marked),
            // then evaluates the gradient terms of the marked entries only, in
            // tile order; the unmarked pairs contribute exactly zero.
            const R lim = hinv * hinv * (R)1.00002;
            auto mark = [&](int k, unsigned &msk) {
                const R4 pj = s_p[wid][k];
                const R dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
                const R r2 = dx * dx + dy * dy + dz * dz;
                if (!(r2 * lim >= (R)1)) msk |= 1u << (k & 31);
            };
            auto run = [&](int head, int n) {
                unsigned msk = 0;
                if (tpi == 1 && n == 32) {
#pragma unroll 8
                    for (int k = 0; k < 32; ++k) mark(head + k, msk);
                } else {
                    for (int k = sub; k < n; k += tpi) mark(head + k, msk);
                }
                while (msk) {
                    const int k = __ffs(msk) - 1;
                    msk &= msk - 1;
                    pair(head + k);
                }
                fold();
                __syncwarp();
            };
            if (nl_ok && __all_sync(FULL, (float)h <= nl_h)) {
                // this lane's list, two entries per round (gathers first)
                const int cmax = (int)__reduce_max_sync(FULL, (unsigned)ncnt);
                for (int c0 = 0; c0 < cmax; c0 += 2) {
                    int jj[2];
                    R4 pj[2];
                    R4 vh[2];
                    float4 vl[2];
                    long long idj[2];
#pragma unroll
                    for (int u = 0; u < 2; ++u) jj[u] = (c0 + u < ncnt) ? a.nbr[nlb + (c0 + u) * 32] : -1;
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        if (jj[u] >= 0) {
                            pj[u] = jpos(jj[u]);
                            if constexpr (F64) {
                                const dbl4 v = a.j_vel[jj[u]];
                                vh[u] = Real<F64>::make4((R)v.x, (R)v.y, (R)v.z, (R)0);
                                vl[u] = make_float4(0, 0, 0, 0);
                            } else {
                                vh[u] = __ldg(&a.fj.vhi[jj[u]]);
                                vl[u] = __ldg(&a.fj.vlo[jj[u]]);
                            }
                            idj[u] = __ldg(&a.j_id[jj[u]]);
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 2; ++u)
                        if (jj[u] >= 0) gpair(pj[u], vh[u].x, vh[u].y, vh[u].z, vl[u].x, vl[u].y, vl[u].z, idj[u]);
                    if ((c0 & 7) == 6) fold();
                }
                fold();
                if (r.act) ev_list_g += (unsigned)ncnt;
                ++n_listed;
            } else {
                sweep(support2<R>(h), true, false, run);
            }
            const double sg = seg_sum(g_acc.value(), tpi);
            const double sd = seg_sum(d_acc.value(), tpi);
            const double sx = seg_sum(rx_acc.value(), tpi);
            const double sy = seg_sum(ry_acc.value(), tpi);
            const double sz = seg_sum(rz_acc.value(), tpi);
            if (r.act && sub == 0) {
                double divv, rotv, omega;
                if (F64) {
                    const double hinv_d = 1.0 / h;
                    const double hinv4 = hinv_d * hinv_d * hinv_d * hinv_d;
                    const double grdh = -hinv4 * sg;
                    const double rx = CEFF1 * hinv4 * sx, ry = CEFF1 * hinv4 * sy, rz = CEFF1 * hinv4 * sz;
                    const double rhoinv = 1.0 / (double)rho;
                    omega = 1.0 / (1.0 + h * rhoinv * grdh / 3.0);
                    const double rot2 = rx * rx + ry * ry + rz * rz;
                    const double rot = (rot2 != 0.0) ? sqrt(rot2) : 0.0;
                    divv = -CEFF1 * hinv4 * sd * rhoinv * omega;
                    rotv = rot * rhoinv * omega;
                } else {
                    const float hf = (float)h;
                    const float hinv_f = 1.0f / hf;
                    const float hinv4 = hinv_f * hinv_f * hinv_f * hinv_f;
                    const float rinv = 1.0f / (float)rho;
                    const float g = -hinv4 * (float)sg;
                    const float xf = (float)CEFF1 * hinv4 * (float)sx, yf = (float)CEFF1 * hinv4 * (float)sy,
                                zf = (float)CEFF1 * hinv4 * (float)sz;
                    const float om = 1.0f / (1.0f + hf * rinv * g / 3.0f);
                    const float rot2 = xf * xf + yf * yf + zf * zf;
                    omega = om;
                    divv = -(float)CEFF1 * hinv4 * (float)sd * rinv * om;
                    rotv = ((rot2 != 0.0f) ? sqrtf(rot2) : 0.0f) * rinv * om;
                }
                a.o_dens[ii] = (double)rho;
                a.o_divv[ii] = divv;
                a.o_rotv[ii] = rotv;
                a.o_grdh[ii] = omega;
                a.o_ksr[ii] = h;
                a.o_np[ii] = (long long)np;
                a.o_itr[ii] = itr ? 1 : 0;
            }
        }
        if (a.n_eval) {
            const unsigned long long l0 = __reduce_add_sync(FULL, ev_list);
            const unsigned long long l1 = __reduce_add_sync(FULL, ev_list_g);
            if (lane == 0) {
                atomicAdd(a.n_eval, (unsigned long long)kept_rho * (unsigned long long)r.ni + l0);
                atomicAdd(a.n_eval + 1, (unsigned long long)(kept - kept_rho) * (unsigned long long)r.ni + l1);
            }
        }
        if (a.n_pass && lane == 0) {
            atomicAdd(a.n_pass, (unsigned long long)n_listed);
            atomicAdd(a.n_pass + 1, (unsigned long long)(3 - n_listed));
        }
    }
}

// Re-walks of few particles (the search-radius loop of hdr_density.hpp:
// 382-414 late in its course: typically a handful of particles whose h
// grew past 1.1^k times its first guess).  density_kernel gives such a walk
// one warp, which streams the walk's list 32 entries at a time and waits on
// every chunk's loads; here one block takes a walk and evaluates its
// iterating particles one after another, every pass spreading the whole
// list over the block's threads.  Same pair terms, per-particle updates,
// search-radius decision, ambiguity queue and outputs as density_kernel
// (for a one-particle item: positions relative to the particle itself);
// each thread sums its entries (FP32C: Kahan) and the block adds the
// threads' sums in FP64.  Runs only when *small is set (the caller then
// leaves density_kernel no items).
constexpr int REWALK_THREADS = 256;
template <int N>
__device__ __forceinline__ void block_sum(double (&v)[N], double (*red)[REWALK_THREADS / 32]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < N; ++q) {
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(FULL, v[q], o);
        if (lane == 0) red[q][wid] = v[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < N; ++q) {
        double t = 0.0;
        for (int u = 0; u < REWALK_THREADS / 32; ++u) t += red[q][u];
        v[q] = t;
    }
    __syncthreads();
}
// Error bits (scal[err_slot]): list_err_mask marks lists that cannot be
// used (a failed build: nothing runs), bounds_bit is raised for an index
// outside the particle or list arrays (that access is skipped).
struct RewalkBounds {
    int n;                 // particles
    long long list_cap;    // entries of the walks' lists
    int *err;              // error word
    int list_err_mask;
    int bounds_bit;
};
template <bool F64>
__global__ void __launch_bounds__(REWALK_THREADS) density_rewalk_blocks(const DensityArgs a, const int *n_walks,
                                                                       const int *seg_first, const int *seg_count,
                                                                       const int *small, RewalkBounds bnd) {
    typedef typename Real<F64>::T R;
    __shared__ double red[6][REWALK_THREADS / 32];
    if (!*small || (*bnd.err & bnd.list_err_mask)) return;
    const int nw = *n_walks;
    const double ksr_max = a.ksr_max_dev ? *a.ksr_max_dev : a.ksr_max;
    for (int w = blockIdx.x; w < nw; w += gridDim.x) {
        const int jb = a.j_off[w], je = a.j_off[w + 1];
        if (jb < 0 || je < jb || (long long)je > bnd.list_cap) {
            if (threadIdx.x == 0) atomicOr(bnd.err, bnd.bounds_bit);
            continue;   // block-uniform
        }
        for (int s = 0; s < seg_count[w]; ++s) {
            const int u = seg_first[w] + s;
            const int ii = (u >= 0 && u < bnd.n) ? a.i_list[u] : -1;
            if (ii < 0 || ii >= bnd.n) {
                if (threadIdx.x == 0) atomicOr(bnd.err, bnd.bounds_bit);
                continue;   // block-uniform
            }
            float4 cph = make_float4(0, 0, 0, 0), cpl = cph;
            dbl4 ci = make_dbl4(0, 0, 0, 0);
            if (F64) ci = a.i_pm[ii];
            else { cph = a.fi.phi[ii]; cpl = a.fi.plo[ii]; }
            // position of j relative to i (FP32C) or absolute (FP64), and its mass
            auto rel = [&](int j, R &dx, R &dy, R &dz) -> R {
                if constexpr (F64) {
                    const dbl4 p = a.j_pm[j];
                    dx = (R)ci.x - (R)p.x; dy = (R)ci.y - (R)p.y; dz = (R)ci.z - (R)p.z;
                    return (R)p.w;
                } else {
                    const float4 ph = a.fj.phi[j], pl = a.fj.plo[j];
                    dx = -df_diff(ph.x, pl.x, cph.x, cpl.x);
                    dy = -df_diff(ph.y, pl.y, cph.y, cpl.y);
                    dz = -df_diff(ph.z, pl.z, cph.z, cpl.z);
                    return (R)ph.w;
                }
            };
            double h = a.i_ksr[ii];
            const double mi = a.i_pm[ii].w;
            R rho = 0;
            long long np = 0;
            // three fixed-point passes, hdr_density.hpp:264-302
            for (int pass = 0; pass < 3; ++pass) {
                const R hinv = (R)1 / (R)h;
                const R hinv2 = hinv * hinv;
                Acc<F64> acc;
                long long cnt = 0;
                for (int k = jb + threadIdx.x; k < je; k += REWALK_THREADS) {
                    const int j = a.j_idx ? a.j_idx[k] : k;
                    if (j < 0 || j >= bnd.n) {
                        atomicOr(bnd.err, bnd.bounds_bit);
                        continue;
                    }
                    R dx, dy, dz;
                    const R m = rel(j, dx, dy, dz);
                    const R q = sqrt_q(dx * dx + dy * dy + dz * dz, hinv2);
                    const R u = max0((R)1 - q);
                    const R u2 = u * u;
                    if (pass == 2) cnt += (q < (R)1) ? 1 : 0;
                    acc.add(m * (u2 * u2 * ((R)1 + (R)4 * q)));
                }
                double v[2] = {acc.value(), (double)cnt};
                block_sum(v, red);
                double hn;
                if (F64) {
                    const double hinv_d = 1.0 / h;
                    rho = (R)(CEFF0 * hinv_d * hinv_d * hinv_d * v[0]);
                    hn = a.eta_ksrh * cbrt(mi / (double)rho);
                } else {
                    const float hinv_f = (float)hinv;
                    const float rho_f = (float)CEFF0 * hinv_f * hinv_f * hinv_f * (float)v[0];
                    rho = (R)rho_f;
                    hn = (double)((float)a.eta_ksrh * cbrtf((float)mi / rho_f));
                }
                hn = (hn < ksr_max) ? hn : ksr_max;
                np = (long long)v[1];
                h = hn;
            }
            // the search-radius decision of the last pass (hdr_density.hpp:299)
            const double rs_i = a.i_rs[ii];
            const bool itr = h > rs_i;
            if (!F64 && a.amb_count && threadIdx.x == 0 && fabs(h - rs_i) <= (double)a.amb_tol * rs_i) {
                const int q = atomicAdd(a.amb_count, 1);
                if (q < a.amb_cap) {
                    a.amb_i[q] = ii;
                    a.amb_w[q] = w;
                }
            }
            // gradient pass with the final h, hdr_density.hpp:304-349
            const long long idi = a.i_id[ii];
            R vxi, vyi, vzi;
            float lxi = 0.0f, lyi = 0.0f, lzi = 0.0f;
            if (F64) {
                const dbl4 vv = a.i_vel[ii];
                vxi = (R)vv.x; vyi = (R)vv.y; vzi = (R)vv.z;
            } else {
                const float4 vh = a.fi.vhi[ii], vl = a.fi.vlo[ii];
                vxi = vh.x; vyi = vh.y; vzi = vh.z;
                lxi = vl.x; lyi = vl.y; lzi = vl.z;
            }
            const R hinv = (R)1 / (R)h;
            Acc<F64> g_acc, d_acc, rx_acc, ry_acc, rz_acc;
            for (int k = jb + threadIdx.x; k < je; k += REWALK_THREADS) {
                const int j = a.j_idx ? a.j_idx[k] : k;
                if (j < 0 || j >= bnd.n) {
                    atomicOr(bnd.err, bnd.bounds_bit);
                    continue;
                }
                R dx, dy, dz;
                const R m = rel(j, dx, dy, dz);
                R ux, uy, uz;
                if constexpr (F64) {
                    const dbl4 vv = a.j_vel[j];
                    ux = vxi - (R)vv.x; uy = vyi - (R)vv.y; uz = vzi - (R)vv.z;
                } else {
                    const float4 vh = a.fj.vhi[j], vl = a.fj.vlo[j];
                    ux = vxi - vh.x; uy = vyi - vh.y; uz = vzi - vh.z;
                    ux += (R)(lxi - vl.x);
                    uy += (R)(lyi - vl.y);
                    uz += (R)(lzi - vl.z);
                }
                const R r2 = dx * dx + dy * dy + dz * dz;
                const R ri = (idi != a.j_id[j]) ? rsqrt_r(r2) : (R)0;
                const R q = r2 * ri * hinv;
                const R u = max0((R)1 - q);
                const R u2 = u * u;
                const R u3 = u2 * u;
                const R p14 = (R)1 + (R)4 * q;
                const R w0 = u2 * u2 * p14;
                const R w1 = w1_term(q, u, u2, u3, p14);
                g_acc.add(m * ((R)(3.0 * CEFF0) * w0 + (R)CEFF1 * q * w1));
                const R dw = m * w1 * ri;
                d_acc.add((ux * dx + uy * dy + uz * dz) * dw);
                rx_acc.add((uy * dz - uz * dy) * dw);
                ry_acc.add((uz * dx - ux * dz) * dw);
                rz_acc.add((ux * dy - uy * dx) * dw);
            }
            double v[5] = {g_acc.value(), d_acc.value(), rx_acc.value(), ry_acc.value(), rz_acc.value()};
            block_sum(v, red);
            if (threadIdx.x == 0) {
                const double sg = v[0], sd = v[1], sx = v[2], sy = v[3], sz = v[4];
                double divv, rotv, omega;
                if (F64) {
                    const double hinv_d = 1.0 / h;
                    const double hinv4 = hinv_d * hinv_d * hinv_d * hinv_d;
                    const double grdh = -hinv4 * sg;
                    const double rx = CEFF1 * hinv4 * sx, ry = CEFF1 * hinv4 * sy, rz = CEFF1 * hinv4 * sz;
                    const double rhoinv = 1.0 / (double)rho;
                    omega = 1.0 / (1.0 + h * rhoinv * grdh / 3.0);
                    const double rot2 = rx * rx + ry * ry + rz * rz;
                    const double rot = (rot2 != 0.0) ? sqrt(rot2) : 0.0;
                    divv = -CEFF1 * hinv4 * sd * rhoinv * omega;
                    rotv = rot * rhoinv * omega;
                } else {
                    const float hf = (float)h;
                    const float hinv_f = 1.0f / hf;
                    const float hinv4 = hinv_f * hinv_f * hinv_f * hinv_f;
                    const float rinv = 1.0f / (float)rho;
                    const float g = -hinv4 * (float)sg;
                    const float xf = (float)CEFF1 * hinv4 * (float)sx, yf = (float)CEFF1 * hinv4 * (float)sy,
                                zf = (float)CEFF1 * hinv4 * (float)sz;
                    const float om = 1.0f / (1.0f + hf * rinv * g / 3.0f);
                    const float rot2 = xf * xf + yf * yf + zf * zf;
                    omega = om;
                    divv = -(float)CEFF1 * hinv4 * (float)sd * rinv * om;
                    rotv = ((rot2 != 0.0f) ? sqrtf(rot2) : 0.0f) * rinv * om;
                }
                a.o_dens[ii] = (double)rho;
                a.o_divv[ii] = divv;
                a.o_rotv[ii] = rotv;
                a.o_grdh[ii] = omega;
                a.o_ksr[ii] = h;
                a.o_np[ii] = np;
                a.o_itr[ii] = itr ? 1 : 0;
            }
        }
    }
}

// ---------------------------------------------------------------- hydro
struct HydroArgs {
    // FP64 mode records
    const dbl4 *i_pm;    // x, y, z, (mass unused)
    const dbl4 *i_vel;
    const dbl4 *i_h1;    // hinv, pres, presc, bswt
    const dbl4 *i_h2;    // dens, vsnd, alph, alphu
    const double2 *i_h3; // thrm, eta
    const dbl4 *j_pm;    // x, y, z, mass
    const dbl4 *j_vel;
    const dbl4 *j_h1;
    const dbl4 *j_h2;
    const double2 *j_h3;
    // FP32C mode records: vhi.w = hinv, vlo.w = hinv^4,
    // g1 = (P_hi, P_lo, presc, bswt), g2 = (dens, vsnd, alph, alphu),
    // g3 = (thrm_hi, thrm_lo, eta, -)
    F32Part fi, fj;
    const float4 *fi_g1, *fi_g2, *fi_g3, *fj_g1, *fj_g2, *fj_g3;
    const long long *i_id;
    const long long *j_id;
    const WorkItem *items;
    int n_items;
    const int *n_items_dev;
    const int *j_off;
    const int *j_idx;
    const int *i_list;
    int *queue;
    // outputs
    double *o_acch;      // 3 per particle
    double *o_accg;      // 3 per particle
    double *o_udot, *o_vsmx, *o_diffu;
    // when set: pair evaluations performed in full (near) and for the
    // signal velocity only (far), j-entries x i-particles
    unsigned long long *n_eval_near, *n_eval_far;
    // when set: per walk, the largest sound speed of its j-list (the signal
    // velocity of every i-particle of the walk is at least its own sound
    // speed plus this), which lets tiles that cannot raise the maximum skip
    // their signal-velocity terms
    const double *walk_csmax = nullptr;
    int sv_skip = 0;   // nonzero: tiles test the bound and skip (0: every term evaluated)
    // when set: [0] 32-entry tiles whose signal-velocity terms were skipped,
    // [1] tiles evaluated
    unsigned long long *n_skip = nullptr;
    // when set: [0] marked pairs (inside either support, evaluated in
    // full), [1] lane slots their loops occupied (per 32-entry tile, 32 x
    // the largest per-lane count)
    unsigned long long *n_mark = nullptr;
    // FP32C: the kernel evaluates the signal velocities and writes, per
    // i-particle, the j indices of its marked pairs (self pairs excluded) to
    // row i of df_list (df_cap entries) and their number to df_cnt[i]; a
    // particle with more than df_cap appends (i, walk) to df_ovf and counts
    // it in *df_novf.  The double-float pass (hydro_df_lists /
    // hydro_df_sweep) then forms acch, accg, udot and diffu.  g4 records:
    // (1/h hi, 1/h lo, h^-4 hi, h^-4 lo).
    const float4 *fi_g4 = nullptr, *fj_g4 = nullptr;
    int *df_list = nullptr;
    int df_cap = 0;
    int *df_cnt = nullptr;
    int2 *df_ovf = nullptr;
    int *df_novf = nullptr;
    int n_i = 0;   // i-particles (the double-float pass covers [0, n_i))
};

// Capacity of a particle's row of marked pairs in the FP32C hydro lists
// (~50-60 marked pairs are typical; a particle whose row overflows is summed
// over its walk's whole list instead).
constexpr int HYDRO_LIST_CAP = 128;
static_assert(HYDRO_LIST_CAP % 4 == 0, "rows of marked pairs start 16-byte aligned");

template <bool F64, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, F64 ? 1 : SPH_HYDRO_MIN_BLOCKS)
hydro_kernel(const HydroArgs a) {
    typedef typename Real<F64>::T R;
    typedef typename Real<F64>::T4 R4;
    // Two 64-entry rings of compacted j records per warp.  Near ring: the
    // j-particles that can lie within the kernel support of some i-particle
    // of the item (r < max(h_i, h_j)), with every field of the pair formula.
    // Far ring: the others, whose pair terms all vanish except the
    // signal-velocity maximum (hdr_hydro.hpp:372 takes it over every j of
    // the list), kept as position + sound speed and velocity only.
    // Near-ring layout (FP32C; FP64 keeps the lo parts at zero):
    __shared__ R4 s_p1[WARPS][64];    // dx, dy, dz (exact hi parts, item frame), hinv
    __shared__ R4 s_p2[WARPS][64];    // position lo parts, vsnd
    __shared__ R4 s_v1[WARPS][64];    // velocity hi, mass
    __shared__ R4 s_v2[WARPS][64];    // velocity lo, hinv^4
    // pair-formula fields (FP64 mode only: FP32C forms the pair sums in a
    // separate double-float pass)
    __shared__ R4 s_c[F64 ? WARPS : 1][64];     // P (hi), presc, bswt, dens
    __shared__ R4 s_d[F64 ? WARPS : 1][64];     // alph, alphu, u (hi), eta
    __shared__ float2 s_f[F64 ? WARPS : 1][64]; // P lo, u lo
    __shared__ long long s_id[WARPS][64];
    __shared__ R4 s_fp[WARPS][64];    // far: centred position, vsnd
    __shared__ R4 s_fv[WARPS][64];    // far: velocity (hi), signal-velocity bound b_j
    __shared__ R s_nb[WARPS][64];     // near: signal-velocity bound b_j
    // FP32C near entries for the mark test: position in the item frame as one
    // float (as the support test has it) and h_j^2 widened by 2e-4; and the
    // entry's j index (written to the marked-pair lists)
    __shared__ float4 s_m[F64 ? 1 : WARPS][64];
    __shared__ int s_jx[F64 ? 1 : WARPS][64];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const unsigned lt = lanemask_lt();
    const int n_items = a.n_items_dev ? *a.n_items_dev : a.n_items;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.queue, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= n_items) return;
        const ItemRef r = decode(a.items[item], a.j_off, a.i_list, lane);
        const int tpi = r.tpi, sub = r.sub, ii = r.ii, nj = r.nj, jb = r.jb;

        R xi, yi, zi, vxi, vyi, vzi, hi_i, hi4_i, pp_i, pc_i, bs_i, dn_i, cs_i, al_i, au_i, eg_i, et_i;
        float lxi = 0.0f, lyi = 0.0f, lzi = 0.0f, plo_i = 0.0f, elo_i = 0.0f;
        float xlo = 0.0f, ylo = 0.0f, zlo = 0.0f;
        float4 cph = make_float4(0, 0, 0, 0), cpl = cph;
        if (F64) {
            const dbl4 p = a.i_pm[ii], v = a.i_vel[ii], h1 = a.i_h1[ii], h2 = a.i_h2[ii];
            const double2 h3 = a.i_h3[ii];
            xi = p.x; yi = p.y; zi = p.z; vxi = v.x; vyi = v.y; vzi = v.z;
            hi_i = h1.x; hi4_i = h1.x * h1.x * h1.x * h1.x; pp_i = h1.y; pc_i = h1.z; bs_i = h1.w;
            dn_i = h2.x; cs_i = h2.y; al_i = h2.z; au_i = h2.w; eg_i = h3.x; et_i = h3.y;
        } else {
            cph = a.fi.phi[r.ic]; cpl = a.fi.plo[r.ic];
            const float4 ph = a.fi.phi[ii], pl = a.fi.plo[ii], vh = a.fi.vhi[ii], vl = a.fi.vlo[ii];
            const float4 g1 = a.fi_g1[ii], g2 = a.fi_g2[ii], g3 = a.fi_g3[ii];
            xi = ph.x - cph.x; yi = ph.y - cph.y; zi = ph.z - cph.z;   // exact hi parts
            xlo = pl.x - cpl.x; ylo = pl.y - cpl.y; zlo = pl.z - cpl.z;
            vxi = vh.x; vyi = vh.y; vzi = vh.z;       // absolute hi/lo, differenced per pair
            lxi = vl.x; lyi = vl.y; lzi = vl.z;
            hi_i = vh.w; hi4_i = vl.w;
            pp_i = g1.x; plo_i = g1.y; pc_i = g1.z; bs_i = g1.w;   // P and u as hi/lo,
            dn_i = g2.x; cs_i = g2.y; al_i = g2.z; au_i = g2.w;    // differenced per pair
            eg_i = g3.x; elo_i = g3.y; et_i = g3.z;
        }
        const long long idi = a.i_id[ii];
        // Signal-velocity bounds.  With v_c the velocity of the item's centre
        // particle, |v_i - v_j| <= d_i + d_j (d = |v - v_c|, FP32C with the
        // hi and lo differences added per component) and |w| <= |v_i - v_j|,
        // so every pair term cs_i + cs_j - 3 min(w, 0) of a tile is at most
        // cs_i + 3 d_i + max_j b_j with b_j = cs_j + 3 d_j.  The maximum over
        // the list starts at cs_i + (largest cs_j of the walk), which no pair
        // term undercuts; a tile whose bound (with a 1e-5 relative margin over
        // the rounding of both) stays below every lane's running maximum adds
        // nothing to it and skips those terms: the maximum is unchanged bit
        // for bit.  The margin also covers the approximate square root of d.
        // Entries beyond both supports are tested as each 32-entry chunk of
        // the list arrives, against the running maximum at that point (which
        // only grows), and are staged in the far ring only when the test
        // fails.
        R vcx, vcy, vcz;
        float lcx = 0.0f, lcy = 0.0f, lcz = 0.0f;
        if (F64) {
            const dbl4 v = a.i_vel[r.ic];
            vcx = v.x; vcy = v.y; vcz = v.z;
        } else {
            const float4 vh = a.fi.vhi[r.ic], vl = a.fi.vlo[r.ic];
            vcx = vh.x; vcy = vh.y; vcz = vh.z;
            lcx = vl.x; lcy = vl.y; lcz = vl.z;
        }
        auto dvel = [&](R hx, R hy, R hz, float lx, float ly, float lz) -> R {
            const R ex = fabs(hx - vcx) + (R)fabsf(lx - lcx);
            const R ey = fabs(hy - vcy) + (R)fabsf(ly - lcy);
            const R ez = fabs(hz - vcz) + (R)fabsf(lz - lcz);
            return sqrt_bound(ex * ex + ey * ey + ez * ez);
        };
        auto sv_bound = [&](R cs, R d) -> R {
            const R b = cs + (R)3 * d;
            return (b < (R)0) ? (R)0 : b;   // NaN stays NaN (no skip)
        };
        const R ub_i = cs_i + (R)3 * dvel(vxi, vyi, vzi, lxi, lyi, lzi);
        // i position in the item frame as one number (box and far pairs)
        const R xc = xi + (R)xlo, yc = yi + (R)ylo, zc = zi + (R)zlo;
        IBox<R> box;
        box.from_lanes(xc, yc, zc);
        const R hm2 = support2<R>(1.0 / (double)hi_i);
        const R hi2_i = hi_i * hi_i;
        const R h2m_i = rcp_r(hi2_i) * (R)1.0002;   // h_i^2 widened as the support test's

        Acc<F64> ax, ay, az, ud, df, gx, gy, gz;
        R vsmx = 0;
        if (a.walk_csmax) {
            const R v0 = cs_i + (R)a.walk_csmax[r.walk];
            vsmx = (v0 > (R)0) ? v0 : (R)0;
        }
        unsigned n_skipped = 0, n_tiles = 0, n_marked = 0, n_slots = 0;
        // true when no pair term with any lane's bound b can exceed any
        // lane's running maximum
        auto below = [&](R b) -> bool {
            R t;
            if constexpr (F64) {
                t = b;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const R u = __shfl_xor_sync(FULL, t, o);
                    t = (u > t || u != u) ? u : t;
                }
            } else {
                // non-negative floats (or NaN) order like their bit patterns
                t = __uint_as_float(__reduce_max_sync(FULL, __float_as_uint(b)));
            }
            const bool ok = (ub_i + t) * (R)1.00001 <= vsmx;
            const bool all = __all_sync(FULL, ok);
            ++n_tiles;
            if (all) ++n_skipped;
            return all;
        };
        // the same for the n-entry ring tile at bound[]
        auto skip_tile = [&](const R *bound, int stride, int n) -> bool {
            if (!a.sv_skip) return false;
            return below((lane < n) ? bound[lane * stride] : (R)0);
        };
        int nhead = 0, nfill = 0, fhead = 0, ffill = 0;
        int lcount = 0;   // FP32C: marked pairs of this lane's particle so far
        long long kept_n = 0, kept_f = 0;
        R pax = 0, pay = 0, paz = 0, pud = 0, pdf = 0, pgx = 0, pgy = 0, pgz = 0;
        // pair separation and velocity difference of near entry k
        auto diffs = [&](int k, R &dx, R &dy, R &dz, R &ux, R &uy, R &uz, R &r2, R &ri) {
            const R4 P1 = s_p1[wid][k];
            const R4 V1 = s_v1[wid][k];
            dx = xi - P1.x; dy = yi - P1.y; dz = zi - P1.z;
            ux = vxi - V1.x; uy = vyi - V1.y; uz = vzi - V1.z;
            if (!F64) {
                const R4 P2 = s_p2[wid][k];
                const R4 V2 = s_v2[wid][k];
                dx += (R)(xlo - (float)P2.x);
                dy += (R)(ylo - (float)P2.y);
                dz += (R)(zlo - (float)P2.z);
                ux += (R)(lxi - (float)V2.x);
                uy += (R)(lyi - (float)V2.y);
                uz += (R)(lzi - (float)V2.z);
            }
            r2 = dx * dx + dy * dy + dz * dz;
            ri = (idi != s_id[wid][k]) ? rsqrt_r(r2) : (R)0;
        };
        // Every near entry: the signal velocity (hdr_hydro.hpp:368-372) and
        // a mark when the pair is inside either support (FP64: r^2
        // min(1/h_i^2, 1/h_j^2) below 1 + 2e-5, so every pair with q_i < 1 or
        // q_j < 1 is marked; FP32C: the test of mark_only below, so that a
        // particle's row holds the same pairs whether or not its tiles skip
        // their signal-velocity terms).  Unmarked pairs add exactly zero to
        // every sum.
        auto signal = [&](int k, unsigned &msk) {
            R dx, dy, dz, ux, uy, uz, r2, ri;
            diffs(k, dx, dy, dz, ux, uy, uz, r2, ri);
            const R w = (dx * ux + dy * uy + dz * uz) * ri;
            const R wneg = w < (R)0 ? w : (R)0;
            const R vs = cs_i + s_p2[wid][k].w - (R)3 * wneg;
            vsmx = vs > vsmx ? vs : vsmx;
            if constexpr (F64) {
                const R hj = s_p1[wid][k].w;
                const R hmin2 = hi2_i < hj * hj ? hi2_i : hj * hj;
                if (!(r2 * hmin2 >= (R)1.00002)) msk |= 1u << (k & 31);
            } else {
                const float4 M = s_m[wid][k];
                const float ex = xc - M.x, ey = yc - M.y, ez = zc - M.z;
                const float lim = h2m_i > M.w ? h2m_i : M.w;
                if (!(ex * ex + ey * ey + ez * ez >= lim)) msk |= 1u << (k & 31);
            }
        };
        // the mark alone (tiles whose signal-velocity terms are skipped).
        // FP32C tests r^2 < max(h_i, h_j)^2 (1 + 2e-4) on the one-float item
        // frame positions of the support test (whose rounding the 2e-4 margin
        // covers), which marks every pair the exact test marks and a few
        // beyond both supports; those add exactly zero (W1 = 0 there).
        auto mark_only = [&](int k, unsigned &msk) {
            if constexpr (!F64) {
                const float4 M = s_m[wid][k];
                const float dx = xc - M.x, dy = yc - M.y, dz = zc - M.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                const float lim = h2m_i > M.w ? h2m_i : M.w;
                if (!(r2 >= lim)) msk |= 1u << (k & 31);
                return;
            }
            const R4 P1 = s_p1[wid][k];
            R dx = xi - P1.x, dy = yi - P1.y, dz = zi - P1.z;
            if (!F64) {
                const R4 P2 = s_p2[wid][k];
                dx += (R)(xlo - (float)P2.x);
                dy += (R)(ylo - (float)P2.y);
                dz += (R)(zlo - (float)P2.z);
            }
            const R r2 = dx * dx + dy * dy + dz * dz;
            const R hj = P1.w;
            const R hmin2 = hi2_i < hj * hj ? hi2_i : hj * hj;
            if (!(r2 * hmin2 >= (R)1.00002)) msk |= 1u << (k & 31);
        };
        // The remaining terms of a marked pair, hdr_hydro.hpp:349-398
        auto pair = [&](int k) {
            R dx, dy, dz, ux, uy, uz, r2, ri;
            diffs(k, dx, dy, dz, ux, uy, uz, r2, ri);
            const R4 P1 = s_p1[wid][k];
            const R4 V1 = s_v1[wid][k];
            const R4 C = s_c[wid][k];
            const R4 D = s_d[wid][k];
            const R hinv4_j = s_v2[wid][k].w;
            const R cs_j = s_p2[wid][k].w;
            R dp = pp_i - C.x, du = eg_i - D.z;
            if (!F64) {
                const float2 F = s_f[wid][k];
                dp += (R)(plo_i - F.x);
                du += (R)(elo_i - F.y);
            }
            const R rr = r2 * ri;
            // kernel gradients W1(q) for both smoothing lengths
            const R qi = rr * hi_i, qj = rr * P1.w;
            const R ui = max0((R)1 - qi), uj = max0((R)1 - qj);
            const R ui2 = ui * ui, uj2 = uj * uj;
            const R w1i = w1_term(qi, ui, ui2, ui2 * ui, (R)1 + (R)4 * qi);
            const R w1j = w1_term(qj, uj, uj2, uj2 * uj, (R)1 + (R)4 * qj);
            const R dw_i = (R)CEFF1 * hi4_i * w1i;
            const R dw_j = (R)CEFF1 * hinv4_j * w1j;
            const R ka = (dw_i + dw_j) * V1.w;
            // viscosity, hdr_hydro.hpp:368-376
            const R w = (dx * ux + dy * uy + dz * uz) * ri;
            const R wneg = w < (R)0 ? w : (R)0;
            const R vs = cs_i + cs_j - (R)3 * wneg;
            const R rhi = rcp_r(dn_i + C.w);
            const R av = (bs_i + C.z) * (al_i + D.x) * vs * wneg;
            // pressure gradient, :378-382
            const R ta = (pc_i + C.y - (R)0.5 * av * rhi) * ka * ri;
            pax -= ta * dx;
            pay -= ta * dy;
            paz -= ta * dz;
            // energy equation with conduction, :384-393
            const R vsu2 = fabs(dp) * rhi * (R)2;
            const R vsu = vsu2 > (R)0 ? vsu2 * rsqrt_r(vsu2) : (R)0;
            pud += ka * (pc_i * w - rhi * ((R)0.25 * av * wneg - (au_i + D.y) * vsu * du));
            pdf += rhi * du * ka * ri;
            // softening correction, :395-398
            const R dg = V1.w * ri * (et_i * dw_i + D.w * dw_j);
            pgx += dg * dx;
            pgy += dg * dy;
            pgz += dg * dz;
        };
        // a j beyond both supports: only the signal velocity (r > 0 here)
        auto far_pair = [&](int k) {
            const R4 P = s_fp[wid][k];
            const R4 V = s_fv[wid][k];
            const R dx = xc - P.x, dy = yc - P.y, dz = zc - P.z;
            const R ux = vxi - V.x, uy = vyi - V.y, uz = vzi - V.z;
            const R r2 = dx * dx + dy * dy + dz * dz;
            const R w = (dx * ux + dy * uy + dz * uz) * rsqrt_r(r2);
            const R wneg = w < (R)0 ? w : (R)0;
            const R vs = cs_i + P.w - (R)3 * wneg;
            vsmx = vs > vsmx ? vs : vsmx;
        };
        auto run_near = [&](int n) {
            pax = 0; pay = 0; paz = 0; pud = 0; pdf = 0; pgx = 0; pgy = 0; pgz = 0;
            unsigned msk = 0;
            if (skip_tile(&s_nb[wid][nhead], 1, n)) {
                if (tpi == 1 && n == 32) {
#pragma unroll HYDRO_MARK_UNROLL
                    for (int k = 0; k < 32; ++k) mark_only(nhead + k, msk);
                } else {
                    for (int k = sub; k < n; k += tpi) mark_only(nhead + k, msk);
                }
            } else if (tpi == 1 && n == 32) {
#pragma unroll 4
                for (int k = 0; k < 32; ++k) signal(nhead + k, msk);
            } else {
                for (int k = sub; k < n; k += tpi) signal(nhead + k, msk);
            }
            if (a.n_mark) {
                const unsigned c = __popc(msk);
                n_marked += c;
                n_slots += 32u * __reduce_max_sync(FULL, c);
            }
            if constexpr (F64) {
                while (msk) {
                    const int k = __ffs(msk) - 1;
                    msk &= msk - 1;
                    pair(nhead + k);
                }
                ax.add(pax);
                ay.add(pay);
                az.add(paz);
                ud.add(pud);
                df.add(pdf);
                gx.add(pgx);
                gy.add(pgy);
                gz.add(pgz);
            } else {
                // append the marked j to the particle's row, self pairs (equal
                // ids, hdr_hydro.hpp:356) dropped; the tpi lanes of one
                // particle write consecutive segments (prefix over the lanes)
                unsigned m = r.act ? msk : 0u;
                for (unsigned t = m; t; t &= t - 1) {
                    const int k = __ffs(t) - 1;
                    if (s_id[wid][nhead + k] == idi) m &= ~(1u << k);
                }
                const int c = __popc(m);
                int incl = c;
                for (int o = 1; o < tpi; o <<= 1) {
                    const int v = __shfl_up_sync(FULL, incl, o, tpi);
                    if (sub >= o) incl += v;
                }
                const int tot = __shfl_sync(FULL, incl, tpi - 1, tpi);
                int pos = lcount + incl - c;
                int *row = a.df_list + (size_t)ii * a.df_cap;
                for (; m; m &= m - 1) {
                    const int k = __ffs(m) - 1;
                    if (pos < a.df_cap) row[pos] = s_jx[wid][nhead + k];
                    ++pos;
                }
                lcount += tot;
            }
            __syncwarp();
        };
        auto run_far = [&](int n) {
            if (skip_tile(&s_fv[wid][fhead].w, 4, n)) {
                __syncwarp();
                return;
            }
            if (tpi == 1 && n == 32) {
#pragma unroll 8
                for (int k = 0; k < 32; ++k) far_pair(fhead + k);
            } else {
                for (int k = sub; k < n; k += tpi) far_pair(fhead + k);
            }
            __syncwarp();
        };
        for (int t = 0; t < nj; t += 32) {
            const int jk = t + lane;
            bool near = false, far = false;
            int j = 0;
            float4 ph, pl, vh, g2;
            dbl4 p64, v64, g1_64, g2_64;
            R px = 0, py = 0, pz = 0, hj_inv = 0, hj2m = 0;
            if (jk < nj) {
                j = a.j_idx ? a.j_idx[jb + jk] : jb + jk;
                if (F64) {
                    p64 = a.j_pm[j];
                    v64 = a.j_vel[j];
                    g1_64 = a.j_h1[j];
                    g2_64 = a.j_h2[j];
                    px = p64.x; py = p64.y; pz = p64.z; hj_inv = g1_64.x;
                } else {
                    ph = a.fj.phi[j];
                    pl = a.fj.plo[j];
                    vh = a.fj.vhi[j];
                    g2 = a.fj_g2[j];
                    px = df_diff(ph.x, pl.x, cph.x, cpl.x);
                    py = df_diff(ph.y, pl.y, cph.y, cpl.y);
                    pz = df_diff(ph.z, pl.z, cph.z, cpl.z);
                    hj_inv = vh.w;
                }
                const R hj = rcp_r(hj_inv);
                const R hj2 = hj * hj * (R)1.0002;
                hj2m = hj2;
                const R rf2 = hj2 > hm2 ? hj2 : hm2;
                near = !(box.d2(px, py, pz) > rf2) || !(hj2 >= (R)0);
                far = !near;
            }
            const unsigned mn = __ballot_sync(FULL, near);
            const unsigned mf = __ballot_sync(FULL, far);
            if (near) {
                const int k = (nhead + nfill + __popc(mn & lt)) & 63;
                if (F64) {
                    const double2 g3 = a.j_h3[j];
                    const double h4 = g1_64.x * g1_64.x * g1_64.x * g1_64.x;
                    s_p1[wid][k] = Real<F64>::make4(p64.x, p64.y, p64.z, g1_64.x);
                    s_p2[wid][k] = Real<F64>::make4(0.0, 0.0, 0.0, g2_64.y);
                    s_v1[wid][k] = Real<F64>::make4(v64.x, v64.y, v64.z, p64.w);
                    s_v2[wid][k] = Real<F64>::make4(0.0, 0.0, 0.0, h4);
                    s_c[wid][k] = Real<F64>::make4(g1_64.y, g1_64.z, g1_64.w, g2_64.x);
                    s_d[wid][k] = Real<F64>::make4(g2_64.z, g2_64.w, g3.x, g3.y);
                    s_f[wid][k] = make_float2(0.0f, 0.0f);
                    s_nb[wid][k] = sv_bound(g2_64.y, dvel(v64.x, v64.y, v64.z, 0.0f, 0.0f, 0.0f));
                } else {
                    // the signal velocity and the mark only: the pair sums are
                    // formed in double-float from the lists (hydro_df_lists)
                    const float4 vl = a.fj.vlo[j];
                    s_p1[wid][k] = Real<F64>::make4((R)(ph.x - cph.x), (R)(ph.y - cph.y), (R)(ph.z - cph.z),
                                                    (R)vh.w);
                    s_p2[wid][k] = Real<F64>::make4((R)(pl.x - cpl.x), (R)(pl.y - cpl.y), (R)(pl.z - cpl.z),
                                                    (R)g2.y);
                    s_v1[wid][k] = Real<F64>::make4((R)vh.x, (R)vh.y, (R)vh.z, (R)ph.w);
                    s_v2[wid][k] = Real<F64>::make4((R)vl.x, (R)vl.y, (R)vl.z, (R)vl.w);
                    s_nb[wid][k] = sv_bound((R)g2.y, dvel(vh.x, vh.y, vh.z, vl.x, vl.y, vl.z));
                    if constexpr (!F64) {
                        s_m[wid][k] = make_float4(px, py, pz, hj2m);
                        s_jx[wid][k] = j;
                    }
                }
                s_id[wid][k] = a.j_id[j];
            }
            // far entries: their signal-velocity bound, and the whole chunk's
            // far entries dropped when none can raise any lane's maximum
            R bfar = 0;
            if (far) {
                if constexpr (F64)
                    bfar = sv_bound(g2_64.y, dvel(v64.x, v64.y, v64.z, 0.0f, 0.0f, 0.0f));
                else
                    bfar = sv_bound((R)g2.y, dvel(vh.x, vh.y, vh.z, lcx, lcy, lcz));
            }
            unsigned ms = mf;
            if (a.sv_skip && mf && below(far ? bfar : (R)0)) ms = 0;
            if (ms & (1u << lane)) {
                const int k = (fhead + ffill + __popc(ms & lt)) & 63;
                if constexpr (F64) {
                    s_fp[wid][k] = Real<F64>::make4(px, py, pz, g2_64.y);
                    s_fv[wid][k] = Real<F64>::make4(v64.x, v64.y, v64.z, bfar);
                } else {
                    s_fp[wid][k] = Real<F64>::make4(px, py, pz, (R)g2.y);
                    s_fv[wid][k] = Real<F64>::make4((R)vh.x, (R)vh.y, (R)vh.z, bfar);
                }
            }
            nfill += __popc(mn);
            ffill += __popc(ms);
            kept_n += __popc(mn);
            kept_f += __popc(mf);
            __syncwarp();
            if (nfill >= 32) {
                run_near(32);
                nhead ^= 32;
                nfill -= 32;
            }
            if (ffill >= 32) {
                run_far(32);
                fhead ^= 32;
                ffill -= 32;
            }
        }
        if (nfill > 0) run_near(nfill);
        if (ffill > 0) run_far(ffill);
        const double svs = seg_max((double)vsmx, tpi);
        if constexpr (F64) {
            const double sax = seg_sum(ax.value(), tpi), say = seg_sum(ay.value(), tpi);
            const double saz = seg_sum(az.value(), tpi), sud = seg_sum(ud.value(), tpi);
            const double sdf = seg_sum(df.value(), tpi), sgx = seg_sum(gx.value(), tpi);
            const double sgy = seg_sum(gy.value(), tpi), sgz = seg_sum(gz.value(), tpi);
            if (r.act && sub == 0) {
                a.o_acch[3 * ii + 0] = 0.5 * sax;
                a.o_acch[3 * ii + 1] = 0.5 * say;
                a.o_acch[3 * ii + 2] = 0.5 * saz;
                a.o_accg[3 * ii + 0] = 0.5 * sgx;
                a.o_accg[3 * ii + 1] = 0.5 * sgy;
                a.o_accg[3 * ii + 2] = 0.5 * sgz;
                a.o_udot[ii] = 0.5 * sud;
                a.o_vsmx[ii] = svs;
                a.o_diffu[ii] = 2.0 * sdf;
            }
        } else if (r.act && sub == 0) {
            a.o_vsmx[ii] = svs;
            a.df_cnt[ii] = lcount;
            if (lcount > a.df_cap) {
                const int e = atomicAdd(a.df_novf, 1);
                a.df_ovf[e] = make_int2(ii, r.walk);
            }
        }
        if (a.n_eval_near && lane == 0) {
            atomicAdd(a.n_eval_near, (unsigned long long)kept_n * (unsigned long long)r.ni);
            atomicAdd(a.n_eval_far, (unsigned long long)kept_f * (unsigned long long)r.ni);
        }
        if (a.n_skip && lane == 0) {
            atomicAdd(a.n_skip, (unsigned long long)n_skipped);
            atomicAdd(a.n_skip + 1, (unsigned long long)n_tiles);
        }
        if (a.n_mark) {
            const unsigned m = __reduce_add_sync(FULL, n_marked);
            if (lane == 0) {
                atomicAdd(a.n_mark, (unsigned long long)m);
                atomicAdd(a.n_mark + 1, (unsigned long long)n_slots);
            }
        }
    }
}

// FP32C hydro, double-float pass over the marked-pair rows: one thread per
// i-particle (particles in index order, so a warp's particles share most of
// their neighbours in L1), two row entries at a time in the two halves of
// packed f32x2 instructions (even and odd entries summed apart and combined
// at the end), an odd last entry alone.  Rows that overflowed are left to
// hydro_df_sweep.
constexpr int HYDRO_DF_THREADS = 128;
__device__ __forceinline__ HydroDFP<float> hydro_df_load(const F32Part &f, const float4 *g1, const float4 *g2,
                                                         const float4 *g3, const float4 *g4, int j) {
    return hydro_df_rec(f.phi[j], f.plo[j], f.vhi[j], f.vlo[j], g1[j], g2[j], g3[j], g4[j]);
}
__device__ __forceinline__ void hydro_df_store(const HydroArgs &a, int p, const HydroDFAcc<float> &acc,
                                               dfk::df presc) {
    double h[3], g[3], ud, dif;
    hydro_df_finish(acc, presc, CEFF1, h, g, &ud, &dif);
    a.o_acch[3 * p + 0] = h[0];
    a.o_acch[3 * p + 1] = h[1];
    a.o_acch[3 * p + 2] = h[2];
    a.o_accg[3 * p + 0] = g[0];
    a.o_accg[3 * p + 1] = g[1];
    a.o_accg[3 * p + 2] = g[2];
    a.o_udot[p] = ud;
    a.o_diffu[p] = dif;
}
__global__ inline void __launch_bounds__(HYDRO_DF_THREADS, SPH_HYDRO_DF_MIN_BLOCKS) hydro_df_lists(const HydroArgs a) {
    using dfk::pk;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n_i; p += gridDim.x * blockDim.x) {
        const int c = a.df_cnt[p];
        if (c > a.df_cap) continue;
        const HydroDFP<float> I = hydro_df_load(a.fi, a.fi_g1, a.fi_g2, a.fi_g3, a.fi_g4, p);
        const HydroDFP<pk> I2 = hydro_df_pack(I, I);
        HydroDFAcc<pk> acc2 = hydro_df_zero<pk>();
        HydroDFAcc<float> acc = hydro_df_zero<float>();
        const int *row = a.df_list + (size_t)p * a.df_cap;
        int k = 0;
        for (; k + 1 < c; k += 2) {
            const HydroDFP<float> J0 = hydro_df_load(a.fj, a.fj_g1, a.fj_g2, a.fj_g3, a.fj_g4, row[k]);
            const HydroDFP<float> J1 = hydro_df_load(a.fj, a.fj_g1, a.fj_g2, a.fj_g3, a.fj_g4, row[k + 1]);
            hydro_df_pair(I2, hydro_df_pack(J0, J1), acc2);
        }
        if (k < c) hydro_df_pair(I, hydro_df_load(a.fj, a.fj_g1, a.fj_g2, a.fj_g3, a.fj_g4, row[k]), acc);
        // (even + odd) + last, each addition renormalised
        dfk::df *v[9] = {&acc.ax, &acc.ay, &acc.az, &acc.gx, &acc.gy, &acc.gz, &acc.ud, &acc.uv, &acc.dif};
        const dfk::dv<pk> *w[9] = {&acc2.ax, &acc2.ay, &acc2.az, &acc2.gx, &acc2.gy, &acc2.gz,
                                   &acc2.ud, &acc2.uv, &acc2.dif};
#pragma unroll
        for (int q = 0; q < 9; ++q) *v[q] = dfk::add(dfk::add(lane0(*w[q]), lane1(*w[q])), *v[q]);
        hydro_df_store(a, p, acc, I.presc);
    }
}

// The same for the particles whose row overflowed: one block per particle
// over its walk's whole j-list (such walks have long lists: a warp alone
// would wait on one load after another), pairs beyond both supports skipped
// (they add exactly zero), the threads' double-float sums combined by warp
// shuffles and then across the warps in a fixed order.
constexpr int HYDRO_SWEEP_THREADS = 512;
__device__ __forceinline__ dfk::df warp_sum_df(dfk::df x) {
    for (int o = 16; o > 0; o >>= 1) {
        const dfk::df y = dfk::make(__shfl_xor_sync(FULL, x.h, o), __shfl_xor_sync(FULL, x.l, o));
        x = dfk::add(x, y);
    }
    return x;
}
__global__ inline void __launch_bounds__(HYDRO_SWEEP_THREADS) hydro_df_sweep(const HydroArgs a) {
    constexpr int NW = HYDRO_SWEEP_THREADS / 32;
    __shared__ dfk::df part[9][NW];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int n_ovf = *a.df_novf;
    for (int e = blockIdx.x; e < n_ovf; e += gridDim.x) {
        const int2 ent = a.df_ovf[e];
        const int p = ent.x, w = ent.y;
        const int jb = a.j_off[w], je = a.j_off[w + 1];
        const long long idi = a.i_id[p];
        const HydroDFP<float> I = hydro_df_load(a.fi, a.fi_g1, a.fi_g2, a.fi_g3, a.fi_g4, p);
        HydroDFAcc<float> acc = hydro_df_zero<float>();
        const float hi2 = 1.0f / (I.hinv.h * I.hinv.h);
        for (int k = jb + threadIdx.x; k < je; k += HYDRO_SWEEP_THREADS) {
            const int j = a.j_idx ? a.j_idx[k] : k;
            if (a.j_id[j] == idi) continue;
            // pairs beyond both supports add exactly zero: skip them on an
            // FP32 distance test with a margin far above its rounding
            const float4 ph = a.fj.phi[j], pl = a.fj.plo[j], vh = a.fj.vhi[j];
            const float dx = (I.xh - ph.x) + (I.xl - pl.x), dy = (I.yh - ph.y) + (I.yl - pl.y);
            const float dz = (I.zh - ph.z) + (I.zl - pl.z);
            const float hj2 = 1.0f / (vh.w * vh.w);
            if (dx * dx + dy * dy + dz * dz > fmaxf(hi2, hj2) * 1.001f) continue;
            hydro_df_pair(I, hydro_df_rec(ph, pl, vh, a.fj.vlo[j], a.fj_g1[j], a.fj_g2[j], a.fj_g3[j], a.fj_g4[j]),
                          acc);
        }
        dfk::df *v[9] = {&acc.ax, &acc.ay, &acc.az, &acc.gx, &acc.gy, &acc.gz, &acc.ud, &acc.uv, &acc.dif};
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const dfk::df t = warp_sum_df(*v[q]);
            if (lane == 0) part[q][wid] = t;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                dfk::df t = part[q][0];
                for (int u = 1; u < NW; ++u) t = dfk::add(t, part[q][u]);
                *v[q] = t;
            }
            hydro_df_store(a, p, acc, I.presc);
        }
        __syncthreads();   // part[] is rewritten by the next particle
    }
}

// ---------------------------------------------------------------- gravity
struct GravityArgs {
    // FP64 mode: i (x, y, z, eps2); j sources split at n_split: index
    // k < n_split reads (j_pm, j_eps2)[k], k >= n_split reads
    // (s_pm, s_eps2)[k - n_split] (superparticles / tree-node monopoles)
    const dbl4 *i_pe;
    const dbl4 *j_pm;       // x, y, z, mass
    const double *j_eps2;
    const dbl4 *s_pm;
    const double *s_eps2;
    // FP32C mode: hi = (x, y, z, mass), lo = (x, y, z, eps2); fi_* for the
    // i-particles, f_* for the j particles and f_s* for the monopoles
    const float4 *fi_phi, *fi_plo, *f_phi, *f_plo, *f_shi, *f_slo;
    int n_split;
    const WorkItem *items;
    int n_items;
    const int *n_items_dev;
    const int *j_off;
    const int *j_idx;
    const int *i_list;
    int *queue;
    double *o_acc;          // 3 per particle (assigned)
    double *o_pot, *o_eta;
    // quadrupole of the sources k >= n_split (tree nodes), traceless, about
    // their centre of mass; null: monopoles only (the reference's SPJ).
    // FP64: 6 per node (xx, yy, zz, xy, xz, yz); FP32C: (xx, yy, zz, xy) and
    // (xz, yz, -, -)
    const double *s_quad;
    const float4 *f_sq0, *f_sq1;
};

// JT: the j-tile, list entries a warp stages in shared memory per pass (32
// or 64; each lane loads JT / 32 of them one tile ahead) and sums in FP32
// before folding into the compensated accumulators.
template <bool F64, int WARPS, int JT = 32>
__global__ void __launch_bounds__(WARPS * 32, F64 ? 1 : SPH_GRAVITY_MIN_BLOCKS)
gravity_kernel(const GravityArgs a) {
    typedef typename Real<F64>::T R;
    typedef typename Real<F64>::T4 R4;
    static_assert(JT == 32 || JT == 64, "j-tile of 32 or 64 entries");
    constexpr int S = JT / 32;        // entries per lane and tile
    constexpr int QR = 64 * S;        // quadrupole ring: < 32 left + a tile
    // FP64: one record per entry; FP32C: structure of arrays, so that two
    // consecutive entries load as one f32x2 operand
    __shared__ R4 s_p[F64 ? WARPS : 1][JT];   // dx, dy, dz, mass
    __shared__ R s_e[F64 ? WARPS : 1][JT];    // eps2
    __shared__ __align__(16) float s_x[F64 ? 1 : WARPS][JT], s_y[F64 ? 1 : WARPS][JT], s_z[F64 ? 1 : WARPS][JT],
        s_m[F64 ? 1 : WARPS][JT], s_q[F64 ? 1 : WARPS][JT];
    // tree-node entries of the list with their quadrupoles, compacted into a
    // ring (position in the item frame + eps^2; Q xx yy zz xy; Q xz yz)
    __shared__ R4 q_p[WARPS][QR];
    __shared__ R4 q_a[WARPS][QR];
    __shared__ typename Real<F64>::T2 q_b[WARPS][QR];
    const unsigned lt = lanemask_lt();
    const bool quad = F64 ? (a.s_quad != nullptr) : (a.f_sq0 != nullptr);
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int n_items = a.n_items_dev ? *a.n_items_dev : a.n_items;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.queue, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= n_items) return;
        const ItemRef r = decode(a.items[item], a.j_off, a.i_list, lane);
        const int tpi = r.tpi, sub = r.sub, ii = r.ii, nj = r.nj, jb = r.jb;

        R xi, yi, zi, e2i;
        float4 ch = make_float4(0, 0, 0, 0), cl = ch;
        if (F64) {
            const dbl4 p = a.i_pe[ii];
            xi = p.x; yi = p.y; zi = p.z; e2i = p.w;
        } else {
            ch = a.fi_phi[r.ic]; cl = a.fi_plo[r.ic];
            const float4 h = a.fi_phi[ii], l = a.fi_plo[ii];
            xi = df_diff(h.x, l.x, ch.x, cl.x);
            yi = df_diff(h.y, l.y, ch.y, cl.y);
            zi = df_diff(h.z, l.z, ch.z, cl.z);
            e2i = l.w;
        }
        Acc<F64> ax, ay, az, pt, et;
        // j records are loaded one tile ahead of their use, list indices
        // two tiles ahead, so that their latency overlaps the pair loop
        auto jlist = [&](int k) -> int { return a.j_idx ? a.j_idx[jb + k] : jb + k; };
        float4 nh[S], nl[S];   // next tile (FP32C)
        dbl4 np64[S];          // next tile (FP64)
        double ne64[S];
        auto load = [&](int s, int j) {
            if constexpr (F64) {
                if (j < a.n_split) {
                    np64[s] = a.j_pm[j];
                    ne64[s] = a.j_eps2[j];
                } else {
                    np64[s] = a.s_pm[j - a.n_split];
                    ne64[s] = a.s_eps2[j - a.n_split];
                }
            } else {
                if (j < a.n_split) {
                    nh[s] = a.f_phi[j];
                    nl[s] = a.f_plo[j];
                } else {
                    nh[s] = a.f_shi[j - a.n_split];
                    nl[s] = a.f_slo[j - a.n_split];
                }
            }
        };
        int jn[S], jnx[S];   // list index two tiles ahead, of the next tile
#pragma unroll
        for (int s = 0; s < S; ++s) {
            nh[s] = make_float4(0, 0, 0, 0);
            nl[s] = nh[s];
            np64[s] = make_dbl4(0, 0, 0, 0);
            ne64[s] = 0.0;
            jn[s] = 0;
            jnx[s] = 0;
            if (32 * s + lane < nj) {
                jnx[s] = jlist(32 * s + lane);
                load(s, jnx[s]);
            }
            if (JT + 32 * s + lane < nj) jn[s] = jlist(JT + 32 * s + lane);
        }
        int qhead = 0, qfill = 0;
        // quadrupole terms of the node entries in the ring: the potential
        // -(1/2) r.Q.r R^5 and acceleration Q r R^5 - (5/2)(r.Q.r) r R^7 with
        // r = x_i - c and R = (r^2 + eps_node^2)^(-1/2), accumulated doubled
        // like the monopole sums (halved once at the end)
        auto run_quad = [&](int n_q) {
            R qax = 0, qay = 0, qaz = 0, qpt = 0;
            auto quad_term = [&](int k) {
                const R4 P = q_p[wid][qhead + k];
                const R4 A = q_a[wid][qhead + k];
                const typename Real<F64>::T2 B = q_b[wid][qhead + k];
                const R dx = xi - P.x, dy = yi - P.y, dz = zi - P.z;
                const R rr = rsqrt_r(dz * dz + (dy * dy + (dx * dx + P.w)));
                const R rr2 = rr * rr;
                const R rr5 = rr2 * rr2 * rr;
                const R rr7 = rr5 * rr2;
                const R qx = A.x * dx + A.w * dy + B.x * dz;
                const R qy = A.w * dx + A.y * dy + B.y * dz;
                const R qz = B.x * dx + B.y * dy + A.z * dz;
                const R rqr = dx * qx + dy * qy + dz * qz;
                const R f = (R)5 * rqr * rr7;
                const R g = (R)2 * rr5;
                // two fused multiply-adds per component
                qax += qx * g;
                qax -= f * dx;
                qay += qy * g;
                qay -= f * dy;
                qaz += qz * g;
                qaz -= f * dz;
                qpt -= rqr * rr5;
            };
            if (tpi == 1 && n_q == 32) {
#pragma unroll 8
                for (int k = 0; k < 32; ++k) quad_term(k);
            } else {
                for (int k = sub; k < n_q; k += tpi) quad_term(k);
            }
            ax.add(qax);
            ay.add(qay);
            az.add(qaz);
            pt.add(qpt);
            __syncwarp();
        };
        for (int t = 0; t < nj; t += JT) {
#pragma unroll
            for (int s = 0; s < S; ++s) {
                const int jk = t + 32 * s + lane;
                const float4 h = nh[s], l = nl[s];
                const dbl4 p64 = np64[s];
                const double e64 = ne64[s];
                const int jcur = jnx[s];
                if (jk + JT < nj) {
                    jnx[s] = jn[s];
                    load(s, jn[s]);
                }
                if (jk + 2 * JT < nj) jn[s] = jlist(jk + 2 * JT);
                if (quad) {
                    const bool node = jk < nj && jcur >= a.n_split;
                    const unsigned mq = __ballot_sync(FULL, node);
                    if (node) {
                        const int slot = (qhead + qfill + __popc(mq & lt)) & (QR - 1);
                        const int nd = jcur - a.n_split;
                        if constexpr (F64) {
                            const double *q = a.s_quad + 6 * (size_t)nd;
                            q_p[wid][slot] = Real<F64>::make4(p64.x, p64.y, p64.z, e64);
                            q_a[wid][slot] = Real<F64>::make4(q[0], q[1], q[2], q[3]);
                            q_b[wid][slot] = Real<F64>::make2(q[4], q[5]);
                        } else {
                            const float4 q0 = a.f_sq0[nd], q1 = a.f_sq1[nd];
                            q_p[wid][slot] = Real<F64>::make4(df_diff(h.x, l.x, ch.x, cl.x),
                                                              df_diff(h.y, l.y, ch.y, cl.y),
                                                              df_diff(h.z, l.z, ch.z, cl.z), l.w);
                            q_a[wid][slot] = q0;
                            q_b[wid][slot] = make_float2(q1.x, q1.y);
                        }
                    }
                    qfill += __popc(mq);
                }
                if (jk < nj) {
                    const int e = 32 * s + lane;
                    if (F64) {
                        s_p[wid][e] = Real<F64>::make4(p64.x, p64.y, p64.z, p64.w);
                        s_e[wid][e] = e64;
                    } else {
                        s_x[wid][e] = df_diff(h.x, l.x, ch.x, cl.x);
                        s_y[wid][e] = df_diff(h.y, l.y, ch.y, cl.y);
                        s_z[wid][e] = df_diff(h.z, l.z, ch.z, cl.z);
                        s_m[wid][e] = h.w;
                        s_q[wid][e] = l.w;
                    }
                }
            }
            __syncwarp();
            const int n = min(JT, nj - t);
            R pax = 0, pay = 0, paz = 0, ppt = 0, pet = 0;
            auto pair = [&](int k) {
                R4 pj;
                R ej;
                if constexpr (F64) {
                    pj = s_p[wid][k];
                    ej = s_e[wid][k];
                } else {
                    pj = Real<F64>::make4(s_x[wid][k], s_y[wid][k], s_z[wid][k], s_m[wid][k]);
                    ej = s_q[wid][k];
                }
                const R dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
                const R r2 = dx * dx + dy * dy + dz * dz;
                const R rei = rsqrt_r(r2 + e2i);
                const R rej = rsqrt_r(r2 + ej);
                const R rei3 = rei * rei * rei;
                const R rej3 = rej * rej * rej;
                const R g = pj.w * (rei3 + rej3);
                ppt -= pj.w * (rei + rej);
                pax -= dx * g;
                pay -= dy * g;
                paz -= dz * g;
                pet += pj.w * rei3;
            };
            if (!F64 && tpi == 1 && n == JT) {
                // full tile, FP32C: two entries per instruction (f32x2); the
                // even and odd entries are summed separately and combined
                // at the end of the tile.  Sums of -x are kept as sums of x
                // and negated once (exact).
                const f2 XI = f2_make((float)xi, (float)xi), YI = f2_make((float)yi, (float)yi);
                const f2 ZI = f2_make((float)zi, (float)zi), EI = f2_make((float)e2i, (float)e2i);
                const f2 NEG = f2_make(-1.0f, -1.0f);
                f2 AX = f2_make(0.0f, 0.0f), AY = AX, AZ = AX, PT = AX, ET = AX;
#pragma unroll GRAVITY_UNROLL
                for (int k = 0; k < JT; k += 2) {
                    const f2 DX = f2_fma(f2_lds(&s_x[wid][k]), NEG, XI);
                    const f2 DY = f2_fma(f2_lds(&s_y[wid][k]), NEG, YI);
                    const f2 DZ = f2_fma(f2_lds(&s_z[wid][k]), NEG, ZI);
                    const f2 M = f2_lds(&s_m[wid][k]);
                    const f2 R2 = f2_fma(DZ, DZ, f2_fma(DY, DY, f2_mul(DX, DX)));
                    const float2 ai = f2_get(f2_add(R2, EI));
                    const float2 aj = f2_get(f2_add(R2, f2_lds(&s_q[wid][k])));
                    const f2 REI = f2_make(rsqrt_r(ai.x), rsqrt_r(ai.y));
                    const f2 REJ = f2_make(rsqrt_r(aj.x), rsqrt_r(aj.y));
                    const f2 REI3 = f2_mul(f2_mul(REI, REI), REI);
                    const f2 REJ3 = f2_mul(f2_mul(REJ, REJ), REJ);
                    const f2 G = f2_mul(M, f2_add(REI3, REJ3));
                    PT = f2_fma(M, f2_add(REI, REJ), PT);
                    AX = f2_fma(DX, G, AX);
                    AY = f2_fma(DY, G, AY);
                    AZ = f2_fma(DZ, G, AZ);
                    ET = f2_fma(M, REI3, ET);
                }
                const float2 ax2 = f2_get(AX), ay2 = f2_get(AY), az2 = f2_get(AZ), pt2 = f2_get(PT), et2 = f2_get(ET);
                pax = -(R)(ax2.x + ax2.y);
                pay = -(R)(ay2.x + ay2.y);
                paz = -(R)(az2.x + az2.y);
                ppt = -(R)(pt2.x + pt2.y);
                pet = (R)(et2.x + et2.y);
            } else if (tpi == 1 && n == JT) {
#pragma unroll 8
                for (int k = 0; k < JT; ++k) pair(k);
            } else {
                for (int k = sub; k < n; k += tpi) pair(k);
            }
            ax.add(pax);
            ay.add(pay);
            az.add(paz);
            pt.add(ppt);
            et.add(pet);
            __syncwarp();
            while (qfill >= 32) {
                run_quad(32);
                qhead = (qhead + 32) & (QR - 1);
                qfill -= 32;
            }
        }
        if (qfill > 0) run_quad(qfill);
        const double sax = seg_sum(ax.value(), tpi), say = seg_sum(ay.value(), tpi);
        const double saz = seg_sum(az.value(), tpi), spt = seg_sum(pt.value(), tpi);
        const double set = seg_sum(et.value(), tpi);
        if (r.act && sub == 0) {
            a.o_acc[3 * ii + 0] = 0.5 * sax;
            a.o_acc[3 * ii + 1] = 0.5 * say;
            a.o_acc[3 * ii + 2] = 0.5 * saz;
            a.o_pot[ii] = 0.5 * spt;
            a.o_eta[ii] = set;
        }
    }
}

// One FP64 work item per queued particle (single-i items use all 32 lanes).
__global__ inline void make_fixup_items(const int *amb_count, const int *amb_w, int cap, WorkItem *items,
                                        int *n_items) {
    const int n = min(*amb_count, cap);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        items[k] = make_int4(amb_w[k], k, 1, 0);
    if (blockIdx.x == 0 && threadIdx.x == 0) *n_items = n;
}

// ---------------------------------------------------------------- records
// Builders of the FP32C double-float records from FP64 arrays (one thread
// per particle).  Each fills hi/lo pairs; aux lanes as documented at the
// consumers above.
__global__ inline void make_density_records(int n, const dbl4 *pm, const dbl4 *vel, float4 *phi, float4 *plo,
                                            float4 *vhi, float4 *vlo) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const dbl4 p = pm[k], v = vel[k];
        const float2 x = df_split(p.x), y = df_split(p.y), z = df_split(p.z);
        const float2 u = df_split(v.x), w = df_split(v.y), s = df_split(v.z);
        phi[k] = make_float4(x.x, y.x, z.x, (float)p.w);
        plo[k] = make_float4(x.y, y.y, z.y, 0.0f);
        vhi[k] = make_float4(u.x, w.x, s.x, 0.0f);
        vlo[k] = make_float4(u.y, w.y, s.y, 0.0f);
    }
}

// Gravity records: hi = (x, y, z, mass), lo = (x, y, z, eps2).
__global__ inline void make_gravity_records(int n, const dbl4 *pm, const double *eps2, float4 *phi, float4 *plo) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const dbl4 p = pm[k];
        const float2 x = df_split(p.x), y = df_split(p.y), z = df_split(p.z);
        phi[k] = make_float4(x.x, y.x, z.x, (float)p.w);
        plo[k] = make_float4(x.y, y.y, z.y, (float)eps2[k]);
    }
}

// The same from (x, y, z, eps2) packs without a mass (gravity i-particles).
__global__ inline void make_gravity_records_pe(int n, const dbl4 *pe, float4 *phi, float4 *plo) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const dbl4 p = pe[k];
        const float2 x = df_split(p.x), y = df_split(p.y), z = df_split(p.z);
        phi[k] = make_float4(x.x, y.x, z.x, 0.0f);
        plo[k] = make_float4(x.y, y.y, z.y, (float)p.w);
    }
}

// Hydro records (layout in hydro_df.cuh): from h1 = (1/h, P, P Omega / rho^2,
// bswt / 2), h2 = (rho, c_s, alpha, alpha_u), h3 = (thrm, eta); 1/h, h^-4 and
// P Omega / rho^2 also as hi/lo splits of their FP64 values.
__global__ inline void make_hydro_records(int n, const dbl4 *pm, const dbl4 *vel, const dbl4 *h1, const dbl4 *h2,
                                          const double2 *h3, float4 *phi, float4 *plo, float4 *vhi, float4 *vlo,
                                          float4 *g1, float4 *g2, float4 *g3, float4 *g4) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const dbl4 p = pm[k], v = vel[k], a = h1[k], b = h2[k];
        const double2 c = h3[k];
        const float2 x = df_split(p.x), y = df_split(p.y), z = df_split(p.z);
        const float2 u = df_split(v.x), w = df_split(v.y), s = df_split(v.z);
        const float2 P = df_split(a.y), T = df_split(c.x), Q = df_split(a.z);
        const double h4d = (a.x * a.x) * (a.x * a.x);
        const float2 H = df_split(a.x), H4 = df_split(h4d), M = df_split(p.w);
        phi[k] = make_float4(x.x, y.x, z.x, M.x);
        plo[k] = make_float4(x.y, y.y, z.y, M.y);
        vhi[k] = make_float4(u.x, w.x, s.x, H.x);
        vlo[k] = make_float4(u.y, w.y, s.y, H4.x);
        g1[k] = make_float4(P.x, P.y, Q.x, (float)a.w);
        g2[k] = make_float4((float)b.x, (float)b.y, (float)b.z, (float)b.w);
        g3[k] = make_float4(T.x, T.y, (float)c.y, Q.y);
        g4[k] = make_float4(H.x, H.y, H4.x, H4.y);
    }
}

}  // namespace sphk
