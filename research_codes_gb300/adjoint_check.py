"""Checks of the bound-mass gradient against central finite differences.

    python -m research_codes_gb300.adjoint_check [--scale 1.0] [--steps 20] [--every 5]
        [--particles 64] [--e0-fraction 0.01 1.0] [--theta 0.5]

The head-on collision of two n=3 polytropes (10 Msun / 4 Rsun each, 2 x 50k
particles at scale 1), K leapfrog steps with checkpoints every `every` steps,
loss sum m sigmoid(-e/e0).  For `particles` seeded random particles and each
of x, y, z, vx, vy, vz: central differences with steps eps = 1e-4 R
(positions) and 1e-4 v_rel (velocities), and again with eps/10.  Where the two
differences disagree by more than 1e-4 the loss is not smooth at that scale (a
tree opening decision or switch change inside the interval) and the point is
reported as non-smooth; elsewhere the adjoint is compared with the eps/10
difference.  theta -> 0 (direct summation: every node is opened) removes the
tree's opening decisions.  The FP32C run's gradient is compared with the FP64
run's.
"""
import argparse
import json
import time

import numpy as np

from . import adjoint, functors, ic
from .system import ParticleSystem, state_from_ic


def head_on(scale, seed=0, vel_noise=0.0):
    """(state, eta, R, v_rel) of the config-3 collision; vel_noise adds random
    velocities (a fraction of v_rel) so that no particle sits on the kinks of
    |div v| and min(w, 0)."""
    s, eta = ic.config_system("c3", scale=scale, seed=seed)
    v_rel = float(np.linalg.norm(s["vel"][0] - s["vel"][-1]))
    R = 4.0e3   # 4 Rsun in code units (1e-3 Rsun)
    s = state_from_ic(s)
    if vel_noise > 0.0:
        s["vel"] = s["vel"] + vel_noise * v_rel * np.random.default_rng(seed + 11).normal(size=s["vel"].shape)
    s["alphu"] = np.zeros(len(s["mass"]))
    return s, eta, R, v_rel


def make_system(precision, n, eta, theta=0.5):
    """A context and system set up as the derivative needs (no clamp of h,
    alpha_u = 0, monopole gravity)."""
    ctx = functors.Context(precision=precision, eta=eta, ksr_max=0.0)
    ps = ParticleSystem(ctx, n, n_group=64, ksr_max_mode=0, alphu_max=0.0, alphu_min=0.0, theta=theta)
    return ctx, ps


def converge_h(ps, s, evals=4):
    """The state's smoothing lengths converged on its positions (the run's
    fixed first guess)."""
    ps.upload(s)
    for _ in range(evals):
        ps.compute_forces()
    out = dict(s)
    out["ksr"] = ps.download("ksr")
    return out


def fd_compare(f, x0, v0, gx, gv, idx, eps_x, eps_v, smooth_tol=1e-4):
    """Central differences of f(x, v) at steps eps and eps/10 for the
    components of particles idx; returns a list of dicts."""
    rows = []
    for i in idx:
        for c in range(6):
            fds = []
            for scale in (1.0, 0.1):
                e = (eps_x if c < 3 else eps_v) * scale
                x, v = x0.copy(), v0.copy()
                arr = x if c < 3 else v
                arr[i, c % 3] += e
                fp = f(x, v)
                arr[i, c % 3] -= 2 * e
                fm = f(x, v)
                fds.append((fp - fm) / (2 * e))
            ad = float((gx if c < 3 else gv)[i, c % 3])
            rows.append({"i": int(i), "c": "xyz"[c % 3] if c < 3 else "v" + "xyz"[c % 3], "fd": fds[1],
                         "fd_coarse": fds[0], "adjoint": ad})
    big = max(abs(r["fd"]) for r in rows) if rows else 0.0
    floor = 1e-3 * big
    for r in rows:
        den = max(abs(r["fd"]), floor)
        r["smooth"] = bool(abs(r["fd"] - r["fd_coarse"]) <= smooth_tol * den)
        r["rel"] = abs(r["adjoint"] - r["fd"]) / den if den > 0 else 0.0
    return rows


def summarise(rows):
    sm = [r["rel"] for r in rows if r["smooth"]]
    return {"components": len(rows), "smooth": len(sm), "max_rel_smooth": max(sm) if sm else None,
            "median_rel_smooth": float(np.median(sm)) if sm else None,
            "max_rel_all": max(r["rel"] for r in rows) if rows else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--every", type=int, default=5)
    ap.add_argument("--particles", type=int, default=64)
    ap.add_argument("--e0-fraction", type=float, nargs="+", default=[0.01, 1.0])
    ap.add_argument("--vel-noise", type=float, default=0.0)
    ap.add_argument("--theta", type=float, default=0.5)
    args = ap.parse_args()
    s, eta, R, v_rel = head_on(args.scale, vel_noise=args.vel_noise)
    n = len(s["mass"])
    out = {"n": n, "steps": args.steps, "every": args.every, "theta": args.theta, "eps_x": 1e-4 * R,
           "eps_v": 1e-4 * v_rel}
    grads = {}
    for prec in ("fp64", "fp32c"):
        ctx, ps = make_system(prec, n, eta, args.theta)
        s0 = converge_h(ps, s)
        run = adjoint.BoundMassRun(ps, s0, steps=args.steps, every=args.every)
        ps.upload(s0)
        ps.compute_forces()
        mean_e = adjoint.energy_scale(ps, 1.0)
        for frac in args.e0_fraction:
            run.e0 = frac * mean_e
            t0 = time.time()
            L = run.forward(s0["pos"], s0["vel"])
            t1 = time.time()
            gx, gv = run.backward()
            t2 = time.time()
            key = f"{prec}_e0_{frac:g}"
            grads[key] = (gx, gv)
            out[key] = {"L": L, "e0": run.e0, "dt": run.dt, "forward_s": t1 - t0, "backward_s": t2 - t1,
                        "grad_norm_x": float(np.linalg.norm(gx)), "grad_norm_v": float(np.linalg.norm(gv))}
            if prec == "fp64" and frac == max(args.e0_fraction):
                idx = np.random.default_rng(5).choice(n, min(args.particles, n), replace=False)
                rows = fd_compare(run.forward, s0["pos"], s0["vel"], gx, gv, idx, 1e-4 * R, 1e-4 * v_rel)
                out[key]["finite_differences"] = summarise(rows)
                out[key]["worst_smooth"] = sorted((r for r in rows if r["smooth"]), key=lambda r: -r["rel"])[:4]
        ps.close()
        ctx.close()
    for frac in args.e0_fraction:
        a, b = grads[f"fp32c_e0_{frac:g}"], grads[f"fp64_e0_{frac:g}"]
        out[f"fp32c_vs_fp64_e0_{frac:g}"] = {
            "x_normwise": float(np.linalg.norm(a[0] - b[0]) / max(np.linalg.norm(b[0]), 1e-300)),
            "v_normwise": float(np.linalg.norm(a[1] - b[1]) / max(np.linalg.norm(b[1]), 1e-300))}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
