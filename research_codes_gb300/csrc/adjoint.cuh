// adjoint.cuh — reverse-mode derivative (vector-Jacobian product) of one
// force evaluation of the particle system: density with the three unrolled
// smoothing-length passes and the gradient pass, EOS and Balsara switch, tree
// gravity (particles and monopole nodes), hydro, and the alpha source.
//
// Given the adjoints (dL/d output) of the evaluation's outputs — total
// acceleration, du/dt, d(alpha)/dt, the final smoothing length h (the next
// evaluation's first guess), and optionally the potential and the density —
// it accumulates the adjoints of its inputs: predicted position and velocity,
// internal energy, alpha, and the first guess of h.  Every formula is the
// derivative of the forward code path (pair_kernels.cuh, system.cu glue):
//
//   density   rho_k = c0 h_k^-3 sum_j m_j W0(r/h_k), h_{k+1} = eta ksrh (m/rho_k)^(1/3),
//             k = 0,1,2; rho = rho_2, h = h_3 (hdr_density.hpp:264-302)
//   gradient  Sg = sum_j m_j (3 c0 W0 + c1 q W1), grdh = -h^-4 Sg,
//             Omega = 1/(1 + h grdh/(3 rho)), D = sum_{j!=i} (u.d) m_j W1/r,
//             R = sum_{j!=i} (u x d) m_j W1/r, divv = -c1 h^-4 D Omega/rho,
//             rotv = c1 h^-4 |R| Omega/rho (hdr_density.hpp:304-349)
//   EOS       P = rho u/1.5, c = sqrt(10 u/9), bswt = |divv|/(|divv|+|rotv|+1e-4 c ksrh/h)
//   gravity   acc = -1/2 sum m (Ri^3+Rj^3) d, pot = -1/2 sum m (Ri+Rj), etas = sum m Ri^3,
//             R = (r^2 + eps^2)^-1/2; nodes carry (centre of mass, mass-weighted eps^2)
//             (hdr_gravity.hpp:286-342); a_g2 = G acc, eta = eps^2 Omega/(3 rho) etas
//   hydro     hdr_hydro.hpp:349-398 with alpha_u = 0 (its channel is then inert)
//   alpha     adot = -(alpha - amin) tau^-1 + max(-divv (amax - alpha), 0),
//             tau^-1 = ksrh c/(4 h) (hdr_hgas.hpp:750-762)
//
// Non-smooth points: away from the kink min(w, 0) and max(., 0) take their
// active branch and |x| its sign; exactly at it (which uniform velocities
// reach: w = 0, div v = 0) the mean of both one-sided derivatives, 1/2 and 0,
// the value central differences converge to.  The lists, tree and time step are those of the
// forward evaluation and are held fixed (the density and hydro kernels are
// C2 at their support, so list membership does not change their values).
// Arithmetic is FP64 throughout; j-side contributions are reduced over the
// warp (whose lanes visit the same list entry) before one atomic add each.
#pragma once

#include "sph_device.cuh"

namespace sphadj {

using sphk::CEFF0;
using sphk::CEFF1;
using sphk::KSRH;
using sphk::FULL;

// One warp's share of a walk: up to 32 consecutive i-particles.
struct AdjItem {
    int walk, first, ni;
};

struct AdjState {
    int n;
    const dbl4 *pos;        // predicted position, mass
    const dbl4 *vel;        // predicted velocity
    const double *uene, *alph, *h0, *h, *dens, *grdh, *divv, *rotv, *pres, *vsnd, *bswt, *eps2, *eta, *etas;
    const dbl4 *mom;        // tree nodes: centre of mass, mass
    const double *neps2;    // tree nodes: mass-weighted eps^2
    const int *parent;      // tree nodes: parent (root: -1); leaf of particle p: n - 1 + p
    const int *d_off, *d_idx, *h_off, *h_idx, *g_off, *g_idx;   // density, hydro, gravity lists per walk
    double G, amax, amin, eta_ksrh;
};

// Seeds (adjoints of the outputs), in sorted particle order.
struct AdjSeed {
    const double *acc;      // 3 per particle
    const double *udot, *adot, *h, *pot, *dens;   // pot / dens may be null
};

// Accumulators, in sorted particle order (zeroed before the first stage).
struct AdjAcc {
    double *x, *v;          // 3 per particle
    double *u, *alph, *h0;  // outputs: internal energy, alpha, first guess of h
    double *h, *rho, *omega, *divv, *rotv, *c, *b, *pc, *eta, *e2, *hinv, *etas, *bswt;
    double *node;           // 4 per tree node: centre of mass (3), eps^2
};

// Wendland C2: W0 = u^4 (1+4q), W1 = -5 q u^3 (the reference's u^4 - u^3 (1+4q)),
// and their q-derivatives, zero for q >= 1.
__device__ __forceinline__ void wendland(double q, double &w0, double &w0p, double &w1, double &w1p) {
    if (q < 1.0) {
        const double u = 1.0 - q, u2 = u * u, u3 = u2 * u;
        w0 = u2 * u2 * (1.0 + 4.0 * q);
        w0p = -20.0 * q * u3;
        w1 = -5.0 * q * u3;
        w1p = -5.0 * u2 * (1.0 - 4.0 * q);
    } else {
        w0 = w0p = w1 = w1p = 0.0;
    }
}

__device__ __forceinline__ double wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

// warp-summed atomic add of a j-side contribution (every lane passes its own
// value, zero where it has none)
__device__ __forceinline__ void wadd(double *p, double v, int lane) {
    v = wsum(v);
    if (lane == 0 && v != 0.0) atomicAdd(p, v);
}

// -------------------------------------------------------------- stage A
// alpha source and the seeds that need no pair loop
__global__ void adj_alpha(AdjState s, AdjSeed sd, AdjAcc a) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
        a.h[i] += sd.h ? sd.h[i] : 0.0;
        if (sd.dens) a.rho[i] += sd.dens[i];
        const double ad = sd.adot[i];
        const double h = s.h[i], c = s.vsnd[i], al = s.alph[i], dv = s.divv[i];
        const double tauinv = 0.25 * KSRH * c / h;
        const double src = -dv * (s.amax - al);
        const double on = src > 0.0 ? 1.0 : (src == 0.0 ? 0.5 : 0.0);
        a.alph[i] += ad * (-tauinv + on * dv);
        a.divv[i] += ad * on * (-(s.amax - al));
        a.c[i] += ad * (-(al - s.amin)) * 0.25 * KSRH / h;
        a.h[i] += ad * (al - s.amin) * tauinv / h;
    }
}

// -------------------------------------------------------------- stage B
// hydro pairs: seeds acch (= acc / 2 per pair sum), accg (= G acc / 2), udot / 2
__global__ void adj_hydro(AdjState s, AdjSeed sd, AdjAcc a, const AdjItem *items, int n_items) {
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = wg; it < n_items; it += nw) {
        const AdjItem t = items[it];
        const bool act = lane < t.ni;
        const int i = t.first + (act ? lane : 0);
        const dbl4 xi = s.pos[i], vi = s.vel[i];
        const double hi = 1.0 / s.h[i], hi4 = hi * hi * hi * hi;
        const double rho_i = s.dens[i], c_i = s.vsnd[i], b_i = 0.5 * s.bswt[i], al_i = s.alph[i];
        const double pc_i = s.pres[i] * s.grdh[i] / (rho_i * rho_i), et_i = s.eta[i];
        const double sc = act ? 1.0 : 0.0;
        const double Ahx = 0.5 * sd.acc[3 * i] * sc, Ahy = 0.5 * sd.acc[3 * i + 1] * sc,
                     Ahz = 0.5 * sd.acc[3 * i + 2] * sc;
        const double Agx = s.G * Ahx, Agy = s.G * Ahy, Agz = s.G * Ahz;
        const double Us = 0.5 * sd.udot[i] * sc;
        double xb[3] = {0, 0, 0}, vb[3] = {0, 0, 0};
        double hinvb = 0, cb = 0, rb = 0, bb = 0, ab = 0, pcb = 0, etb = 0;
        const double hmax_i = s.h[i];
        for (int k = s.h_off[t.walk]; k < s.h_off[t.walk + 1]; ++k) {
            const int j = s.h_idx[k];
            const dbl4 xj = s.pos[j];
            const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double hj_len = s.h[j];
            const double hm = hmax_i > hj_len ? hmax_i : hj_len;
            const bool in = act && j != i && r2 < hm * hm;
            double jx[3] = {0, 0, 0}, jv[3] = {0, 0, 0};
            double jhinv = 0, jc = 0, jr = 0, jb = 0, ja = 0, jpc = 0, jet = 0;
            if (in) {
                const dbl4 vj = s.vel[j];
                const double mj = xj.w;
                const double hj = 1.0 / hj_len, hj4 = hj * hj * hj * hj;
                const double rho_j = s.dens[j], c_j = s.vsnd[j], b_j = 0.5 * s.bswt[j], al_j = s.alph[j];
                const double pc_j = s.pres[j] * s.grdh[j] / (rho_j * rho_j), et_j = s.eta[j];
                const double ux = vi.x - vj.x, uy = vi.y - vj.y, uz = vi.z - vj.z;
                const double ri = 1.0 / sqrt(r2), r = r2 * ri;
                const double qi = r * hi, qj = r * hj;
                double w0, w0p, w1i, w1pi, w1j, w1pj;
                wendland(qi, w0, w0p, w1i, w1pi);
                wendland(qj, w0, w0p, w1j, w1pj);
                const double dWi = CEFF1 * hi4 * w1i, dWj = CEFF1 * hj4 * w1j;
                const double ka = (dWi + dWj) * mj;
                const double w = (dx * ux + dy * uy + dz * uz) * ri;
                const double wn = w < 0.0 ? w : 0.0;
                const double vs = c_i + c_j - 3.0 * wn;
                const double rh = 1.0 / (rho_i + rho_j);
                const double B = b_i + b_j, A = al_i + al_j;
                const double av = B * A * vs * wn;
                const double T = pc_i + pc_j - 0.5 * av * rh;
                const double ta = T * ka * ri;
                const double dg = mj * ri * (et_i * dWi + et_j * dWj);
                // reverse
                const double tab = -(Ahx * dx + Ahy * dy + Ahz * dz);
                double ddx = -ta * Ahx, ddy = -ta * Ahy, ddz = -ta * Ahz;
                const double dgb = Agx * dx + Agy * dy + Agz * dz;
                ddx += dg * Agx; ddy += dg * Agy; ddz += dg * Agz;
                double kab = Us * (pc_i * w - 0.25 * rh * av * wn);
                pcb += Us * ka * w;
                double wb = Us * ka * pc_i;
                double rhb = -Us * ka * 0.25 * av * wn;
                double avb = -Us * ka * 0.25 * rh * wn;
                double wnb = -Us * ka * 0.25 * rh * av;
                const double Tb = tab * ka * ri;
                kab += tab * T * ri;
                double rib = tab * T * ka;
                pcb += Tb;
                jpc = Tb;
                avb += -0.5 * rh * Tb;
                rhb += -0.5 * av * Tb;
                rib += dgb * mj * (et_i * dWi + et_j * dWj);
                etb += dgb * mj * ri * dWi;
                jet = dgb * mj * ri * dWj;
                double dWib = dgb * mj * ri * et_i, dWjb = dgb * mj * ri * et_j;
                bb += avb * A * vs * wn;
                jb = avb * A * vs * wn;
                ab += avb * B * vs * wn;
                ja = avb * B * vs * wn;
                const double vsb = avb * B * A * wn;
                wnb += avb * B * A * vs;
                cb += vsb;
                jc = vsb;
                wnb += -3.0 * vsb;
                if (w < 0.0) wb += wnb;
                else if (w == 0.0) wb += 0.5 * wnb;
                ddx += wb * ri * ux; ddy += wb * ri * uy; ddz += wb * ri * uz;
                const double ubx = wb * ri * dx, uby = wb * ri * dy, ubz = wb * ri * dz;
                rib += wb * (dx * ux + dy * uy + dz * uz);
                rb += -rhb * rh * rh;
                jr = -rhb * rh * rh;
                dWib += kab * mj;
                dWjb += kab * mj;
                // dW = c1 hinv^4 W1(r hinv)
                hinvb += dWib * CEFF1 * (4.0 * hi * hi * hi * w1i + hi4 * w1pi * r);
                jhinv = dWjb * CEFF1 * (4.0 * hj * hj * hj * w1j + hj4 * w1pj * r);
                const double rb_ = dWib * CEFF1 * hi4 * w1pi * hi + dWjb * CEFF1 * hj4 * w1pj * hj;
                const double r2b = 0.5 * rb_ * ri - 0.5 * rib * ri * ri * ri;
                ddx += 2.0 * r2b * dx; ddy += 2.0 * r2b * dy; ddz += 2.0 * r2b * dz;
                xb[0] += ddx; xb[1] += ddy; xb[2] += ddz;
                jx[0] = -ddx; jx[1] = -ddy; jx[2] = -ddz;
                vb[0] += ubx; vb[1] += uby; vb[2] += ubz;
                jv[0] = -ubx; jv[1] = -uby; jv[2] = -ubz;
            }
            if (__any_sync(FULL, in)) {
                for (int c = 0; c < 3; ++c) {
                    wadd(&a.x[3 * j + c], jx[c], lane);
                    wadd(&a.v[3 * j + c], jv[c], lane);
                }
                wadd(&a.hinv[j], jhinv, lane);
                wadd(&a.c[j], jc, lane);
                wadd(&a.rho[j], jr, lane);
                wadd(&a.b[j], jb, lane);
                wadd(&a.alph[j], ja, lane);
                wadd(&a.pc[j], jpc, lane);
                wadd(&a.eta[j], jet, lane);
            }
        }
        if (act) {
            for (int c = 0; c < 3; ++c) {
                atomicAdd(&a.x[3 * i + c], xb[c]);
                atomicAdd(&a.v[3 * i + c], vb[c]);
            }
            atomicAdd(&a.hinv[i], hinvb);
            atomicAdd(&a.c[i], cb);
            atomicAdd(&a.rho[i], rb);
            atomicAdd(&a.b[i], bb);
            atomicAdd(&a.alph[i], ab);
            atomicAdd(&a.pc[i], pcb);
            atomicAdd(&a.eta[i], etb);
        }
    }
}

// -------------------------------------------------------------- stage C
// hydro inputs: hinv = 1/h, presc = P Omega/rho^2, b = bswt/2,
// eta = eps^2 Omega etas/(3 rho), P = rho u/1.5
__global__ void adj_hydro_prep(AdjState s, AdjAcc a) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
        const double h = s.h[i], rho = s.dens[i], P = s.pres[i], om = s.grdh[i], e2 = s.eps2[i];
        const double et = s.etas[i], u = s.uene[i];
        a.h[i] += -a.hinv[i] / (h * h);
        const double pcb = a.pc[i];
        double Pb = pcb * om / (rho * rho);
        a.omega[i] += pcb * P / (rho * rho);
        a.rho[i] += -2.0 * pcb * P * om / (rho * rho * rho);
        a.bswt[i] += 0.5 * a.b[i];
        const double etb = a.eta[i];
        a.e2[i] += etb * om * et / (3.0 * rho);
        a.omega[i] += etb * e2 * et / (3.0 * rho);
        a.rho[i] += -etb * e2 * om * et / (3.0 * rho * rho);
        a.etas[i] = etb * e2 * om / (3.0 * rho);
        a.rho[i] += Pb * u / 1.5;
        a.u[i] += Pb * rho / 1.5;
    }
}

// -------------------------------------------------------------- stage D
// gravity pairs: seeds acc_sum (G acc), pot_sum (G pot), etas
__global__ void adj_gravity(AdjState s, AdjSeed sd, AdjAcc a, const AdjItem *items, int n_items) {
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int n = s.n;
    for (int it = wg; it < n_items; it += nw) {
        const AdjItem t = items[it];
        const bool act = lane < t.ni;
        const int i = t.first + (act ? lane : 0);
        const dbl4 xi = s.pos[i];
        const double e2i = s.eps2[i];
        const double sc = act ? 1.0 : 0.0;
        const double Cx = s.G * sd.acc[3 * i] * sc, Cy = s.G * sd.acc[3 * i + 1] * sc,
                     Cz = s.G * sd.acc[3 * i + 2] * sc;
        const double Pb = sd.pot ? s.G * sd.pot[i] * sc : 0.0;
        const double Eb = a.etas[i] * sc;
        double xb0 = 0, xb1 = 0, xb2 = 0, e2b = 0;
        for (int k = s.g_off[t.walk]; k < s.g_off[t.walk + 1]; ++k) {
            const int j = s.g_idx[k];
            const bool node = j >= n;
            const dbl4 xj = node ? s.mom[j - n] : s.pos[j];
            const double e2j = node ? s.neps2[j - n] : s.eps2[j];
            const double mj = xj.w;
            const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double Ri = 1.0 / sqrt(r2 + e2i), Rj = 1.0 / sqrt(r2 + e2j);
            const double Ri2 = Ri * Ri, Rj2 = Rj * Rj;
            const double g = 0.5 * mj * (Ri2 * Ri + Rj2 * Rj);
            const double gb = -(Cx * dx + Cy * dy + Cz * dz);
            double ddx = -g * Cx, ddy = -g * Cy, ddz = -g * Cz;
            const double Rib = gb * 1.5 * mj * Ri2 - 0.5 * mj * Pb + 3.0 * mj * Ri2 * Eb;
            const double Rjb = gb * 1.5 * mj * Rj2 - 0.5 * mj * Pb;
            const double aib = -0.5 * Rib * Ri2 * Ri, ajb = -0.5 * Rjb * Rj2 * Rj;
            const double r2b = aib + ajb;
            ddx += 2.0 * r2b * dx; ddy += 2.0 * r2b * dy; ddz += 2.0 * r2b * dz;
            xb0 += ddx; xb1 += ddy; xb2 += ddz;
            e2b += aib;
            const bool self = !node && j == i;
            if (self) e2b += ajb;   // eps_j is eps_i
            const double jxb0 = self ? 0.0 : -ddx, jxb1 = self ? 0.0 : -ddy, jxb2 = self ? 0.0 : -ddz;
            const double je2b = self ? 0.0 : ajb;
            if (self) {
                xb0 -= ddx; xb1 -= ddy; xb2 -= ddz;   // d = 0 identically for the self pair
            }
            if (node) {
                double *nb = a.node + 4 * (size_t)(j - n);
                wadd(nb + 0, jxb0, lane);
                wadd(nb + 1, jxb1, lane);
                wadd(nb + 2, jxb2, lane);
                wadd(nb + 3, je2b, lane);
            } else {
                wadd(&a.x[3 * j + 0], jxb0, lane);
                wadd(&a.x[3 * j + 1], jxb1, lane);
                wadd(&a.x[3 * j + 2], jxb2, lane);
                wadd(&a.e2[j], je2b, lane);
            }
        }
        if (act) {
            atomicAdd(&a.x[3 * i + 0], xb0);
            atomicAdd(&a.x[3 * i + 1], xb1);
            atomicAdd(&a.x[3 * i + 2], xb2);
            atomicAdd(&a.e2[i], e2b);
        }
    }
}

// -------------------------------------------------------------- stage E
// node moments to particles: centre = sum m x / M, eps^2 = sum m eps^2 / M,
// so particle p receives m_p sum over the nodes containing it of node_adj / M
__global__ void adj_nodes(AdjState s, AdjAcc a) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < s.n; p += gridDim.x * blockDim.x) {
        double sx = 0, sy = 0, sz = 0, se = 0;
        for (int v = s.n - 1 + p; v >= 0; v = s.parent[v]) {
            const double *nb = a.node + 4 * (size_t)v;
            const double inv = 1.0 / s.mom[v].w;
            sx += nb[0] * inv; sy += nb[1] * inv; sz += nb[2] * inv; se += nb[3] * inv;
        }
        const double m = s.pos[p].w;
        a.x[3 * p] += m * sx;
        a.x[3 * p + 1] += m * sy;
        a.x[3 * p + 2] += m * sz;
        a.e2[p] += m * se;
    }
}

// -------------------------------------------------------------- stage F
// eps^2 = (h/ksrh)^2, Balsara switch, sound speed c = sqrt(10 u/9)
__global__ void adj_switch(AdjState s, AdjAcc a) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
        const double h = s.h[i], c = s.vsnd[i];
        a.h[i] += a.e2[i] * 2.0 * h / (KSRH * KSRH);
        const double dv = s.divv[i], rv = s.rotv[i];
        const double ad = fabs(dv), ar = fabs(rv);
        const double k = 1e-4 * KSRH;
        const double S = ad + ar + k * c / h;
        const double bb = a.bswt[i];
        if (S > 0.0 && bb != 0.0) {
            const double iS2 = 1.0 / (S * S);
            a.divv[i] += bb * (S - ad) * iS2 * (dv < 0.0 ? -1.0 : (dv > 0.0 ? 1.0 : 0.0));
            a.rotv[i] += bb * (-ad * iS2) * (rv < 0.0 ? -1.0 : (rv > 0.0 ? 1.0 : 0.0));
            a.c[i] += bb * (-ad * iS2) * k / h;
            a.h[i] += bb * (-ad * iS2) * (-k * c / (h * h));
        }
        if (c > 0.0) a.u[i] += a.c[i] * 5.0 / (9.0 * c);
    }
}

// -------------------------------------------------------------- stage G
// density gradient pass (final h): Omega, divv, rotv -> positions, velocities, h, rho
__global__ void adj_density_grad(AdjState s, AdjAcc a, const AdjItem *items, int n_items) {
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = wg; it < n_items; it += nw) {
        const AdjItem t = items[it];
        const bool act = lane < t.ni;
        const int i = t.first + (act ? lane : 0);
        const dbl4 xi = s.pos[i], vi = s.vel[i];
        const double h = s.h[i], hinv = 1.0 / h, rho = s.dens[i];
        const int kb = s.d_off[t.walk], ke = s.d_off[t.walk + 1];
        // forward sums
        double Sg = 0, D = 0, Rx = 0, Ry = 0, Rz = 0;
        for (int k = kb; k < ke; ++k) {
            const int j = s.d_idx[k];
            const dbl4 xj = s.pos[j];
            const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 < h * h)) continue;
            const double r = sqrt(r2), q = r * hinv;
            double w0, w0p, w1, w1p;
            wendland(q, w0, w0p, w1, w1p);
            Sg += xj.w * (3.0 * CEFF0 * w0 + CEFF1 * q * w1);
            if (j == i) continue;
            const dbl4 vj = s.vel[j];
            const double ux = vi.x - vj.x, uy = vi.y - vj.y, uz = vi.z - vj.z;
            const double ph = xj.w * w1 / r;
            D += (ux * dx + uy * dy + uz * dz) * ph;
            Rx += (uy * dz - uz * dy) * ph;
            Ry += (uz * dx - ux * dz) * ph;
            Rz += (ux * dy - uy * dx) * ph;
        }
        const double h4i = hinv * hinv * hinv * hinv;
        const double grdh = -h4i * Sg;
        const double Z = 1.0 + h * grdh / (3.0 * rho);
        const double om = 1.0 / Z;
        const double Rn = sqrt(Rx * Rx + Ry * Ry + Rz * Rz);
        double hb = 0, rb = 0;
        const double dvb = act ? a.divv[i] : 0.0, rvb = act ? a.rotv[i] : 0.0;
        const double Db = dvb * (-CEFF1 * h4i * om / rho);
        double omb = (act ? a.omega[i] : 0.0) + dvb * (-CEFF1 * h4i * D / rho) + rvb * CEFF1 * h4i * Rn / rho;
        rb += dvb * CEFF1 * h4i * D * om / (rho * rho) - rvb * CEFF1 * h4i * Rn * om / (rho * rho);
        hb += dvb * 4.0 * CEFF1 * h4i * hinv * D * om / rho - rvb * 4.0 * CEFF1 * h4i * hinv * Rn * om / rho;
        const double rs = Rn > 0.0 ? rvb * CEFF1 * h4i * om / rho / Rn : 0.0;
        const double Rbx = rs * Rx, Rby = rs * Ry, Rbz = rs * Rz;
        const double Zb = -omb * om * om;
        hb += Zb * grdh / (3.0 * rho);
        const double grb = Zb * h / (3.0 * rho);
        rb += -Zb * h * grdh / (3.0 * rho * rho);
        const double Sgb = -grb * h4i;
        hb += grb * 4.0 * h4i * hinv * Sg;
        // pairs
        double xb0 = 0, xb1 = 0, xb2 = 0, vb0 = 0, vb1 = 0, vb2 = 0;
        for (int k = kb; k < ke; ++k) {
            const int j = s.d_idx[k];
            const dbl4 xj = s.pos[j];
            const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const double r2 = dx * dx + dy * dy + dz * dz;
            const bool in = act && j != i && r2 < h * h;
            double jx0 = 0, jx1 = 0, jx2 = 0, jv0 = 0, jv1 = 0, jv2 = 0;
            if (in) {
                const dbl4 vj = s.vel[j];
                const double ux = vi.x - vj.x, uy = vi.y - vj.y, uz = vi.z - vj.z;
                const double r = sqrt(r2), ri = 1.0 / r, q = r * hinv;
                double w0, w0p, w1, w1p;
                wendland(q, w0, w0p, w1, w1p);
                const double m = xj.w;
                const double ph = m * w1 * ri;
                double qb = Sgb * m * (3.0 * CEFF0 * w0p + CEFF1 * (w1 + q * w1p));
                const double ud = ux * dx + uy * dy + uz * dz;
                // D: (u.d) ph
                double ubx = Db * ph * dx, uby = Db * ph * dy, ubz = Db * ph * dz;
                double ddx = Db * ph * ux, ddy = Db * ph * uy, ddz = Db * ph * uz;
                double phb = Db * ud;
                // R: (u x d) ph
                const double cx = uy * dz - uz * dy, cy = uz * dx - ux * dz, cz = ux * dy - uy * dx;
                ubx += ph * (dy * Rbz - dz * Rby);
                uby += ph * (dz * Rbx - dx * Rbz);
                ubz += ph * (dx * Rby - dy * Rbx);
                ddx += ph * (Rby * uz - Rbz * uy);
                ddy += ph * (Rbz * ux - Rbx * uz);
                ddz += ph * (Rbx * uy - Rby * ux);
                phb += Rbx * cx + Rby * cy + Rbz * cz;
                qb += phb * m * w1p * ri;
                const double rib = phb * m * w1;
                const double rbar = qb * hinv;
                hb += -qb * r * hinv * hinv;
                const double r2b = 0.5 * rbar * ri - 0.5 * rib * ri * ri * ri;
                ddx += 2.0 * r2b * dx; ddy += 2.0 * r2b * dy; ddz += 2.0 * r2b * dz;
                xb0 += ddx; xb1 += ddy; xb2 += ddz;
                vb0 += ubx; vb1 += uby; vb2 += ubz;
                jx0 = -ddx; jx1 = -ddy; jx2 = -ddz;
                jv0 = -ubx; jv1 = -uby; jv2 = -ubz;
            }
            if (__any_sync(FULL, in)) {
                wadd(&a.x[3 * j + 0], jx0, lane);
                wadd(&a.x[3 * j + 1], jx1, lane);
                wadd(&a.x[3 * j + 2], jx2, lane);
                wadd(&a.v[3 * j + 0], jv0, lane);
                wadd(&a.v[3 * j + 1], jv1, lane);
                wadd(&a.v[3 * j + 2], jv2, lane);
            }
        }
        if (act) {
            atomicAdd(&a.x[3 * i + 0], xb0);
            atomicAdd(&a.x[3 * i + 1], xb1);
            atomicAdd(&a.x[3 * i + 2], xb2);
            atomicAdd(&a.v[3 * i + 0], vb0);
            atomicAdd(&a.v[3 * i + 1], vb1);
            atomicAdd(&a.v[3 * i + 2], vb2);
            atomicAdd(&a.h[i], hb);
            atomicAdd(&a.rho[i], rb);
        }
    }
}

// -------------------------------------------------------------- stage H
// the three smoothing-length passes: (rho_2, h_3) -> positions, first guess h_0
__global__ void adj_density_passes(AdjState s, AdjAcc a, const AdjItem *items, int n_items) {
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = wg; it < n_items; it += nw) {
        const AdjItem t = items[it];
        const bool act = lane < t.ni;
        const int i = t.first + (act ? lane : 0);
        const dbl4 xi = s.pos[i];
        const int kb = s.d_off[t.walk], ke = s.d_off[t.walk + 1];
        // forward: h_k, rho_k and S'_k = sum m q W0'(q) per pass
        double hk[4], rk[3], sp[3];
        hk[0] = s.h0[i];
        for (int p = 0; p < 3; ++p) {
            const double hinv = 1.0 / hk[p];
            double S0 = 0, S1 = 0;
            for (int k = kb; k < ke; ++k) {
                const int j = s.d_idx[k];
                const dbl4 xj = s.pos[j];
                const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (!(r2 < hk[p] * hk[p])) continue;
                const double q = sqrt(r2) * hinv;
                double w0, w0p, w1, w1p;
                wendland(q, w0, w0p, w1, w1p);
                S0 += xj.w * w0;
                S1 += xj.w * q * w0p;
            }
            rk[p] = CEFF0 * hinv * hinv * hinv * S0;
            sp[p] = S1;
            hk[p + 1] = s.eta_ksrh * cbrt(xi.w / rk[p]);
        }
        // reverse over the scalars
        double rhob[3], hb[4];
        hb[3] = act ? a.h[i] : 0.0;
        rhob[2] = (act ? a.rho[i] : 0.0) + hb[3] * (-hk[3] / (3.0 * rk[2]));
        for (int p = 2; p >= 0; --p) {
            const double hinv = 1.0 / hk[p];
            // rho = c0 h^-3 S0(h): d rho/d h = -3 rho/h - c0 h^-4 sum m q W0'(q)
            hb[p] = rhob[p] * (-3.0 * rk[p] * hinv - CEFF0 * hinv * hinv * hinv * hinv * sp[p]);
            if (p > 0) rhob[p - 1] = hb[p] * (-hk[p] / (3.0 * rk[p - 1]));
        }
        // pairs: d rho_k / d r = c0 h_k^-4 m W0'(q_k)
        double xb0 = 0, xb1 = 0, xb2 = 0;
        const double hmx = fmax(fmax(hk[0], hk[1]), hk[2]);
        for (int k = kb; k < ke; ++k) {
            const int j = s.d_idx[k];
            const dbl4 xj = s.pos[j];
            const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const double r2 = dx * dx + dy * dy + dz * dz;
            const bool in = act && j != i && r2 < hmx * hmx;
            double f = 0.0;
            if (in) {
                const double r = sqrt(r2), ri = 1.0 / r;
                for (int p = 0; p < 3; ++p) {
                    const double hinv = 1.0 / hk[p];
                    double w0, w0p, w1, w1p;
                    wendland(r * hinv, w0, w0p, w1, w1p);
                    f += rhob[p] * CEFF0 * hinv * hinv * hinv * hinv * xj.w * w0p;
                }
                f *= ri;   // r-bar / r, times d for the separation
                xb0 += f * dx; xb1 += f * dy; xb2 += f * dz;
            }
            if (__any_sync(FULL, in)) {
                wadd(&a.x[3 * j + 0], -f * dx, lane);
                wadd(&a.x[3 * j + 1], -f * dy, lane);
                wadd(&a.x[3 * j + 2], -f * dz, lane);
            }
        }
        if (act) {
            atomicAdd(&a.x[3 * i + 0], xb0);
            atomicAdd(&a.x[3 * i + 1], xb1);
            atomicAdd(&a.x[3 * i + 2], xb2);
            a.h0[i] = hb[0];
        }
    }
}

// work items: one per 32 i-particles of a group (offsets from an exclusive
// scan of the per-group counts)
__global__ void adj_item_counts(int n_groups, const int *gcount, int *cnt) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n_groups; g += gridDim.x * blockDim.x)
        cnt[g] = (gcount[g] + 31) / 32;
}
__global__ void adj_fill_items(int n_groups, const int *gfirst, const int *gcount, const int *off, AdjItem *items) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n_groups; g += gridDim.x * blockDim.x) {
        const int c = gcount[g];
        for (int k = 0; 32 * k < c; ++k) {
            AdjItem t;
            t.walk = g;
            t.first = gfirst[g] + 32 * k;
            t.ni = min(32, c - 32 * k);
            items[off[g] + k] = t;
        }
    }
}

}  // namespace sphadj
