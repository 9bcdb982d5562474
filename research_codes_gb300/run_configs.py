"""Runs of the benchmark configurations beyond the headline bench.

    python -m research_codes_gb300.run_configs c1 [--scale 1.0] [--steps 200]
    python -m research_codes_gb300.run_configs c4 [--scale 1.0] [--steps 5]

c1: the head-on collision of two n=3 polytropes (2 x 100k), run for `steps`
    steps with FP32C pair arithmetic and with the plain FP64 kernels from the
    same initial state; per-field relative differences at the end (positions,
    velocities, density, internal energy, acceleration; per particle
    |d| / max(|ref|, 1e-3 max|ref|)) and the energy drift of each run
    (E_total after the run against before, and per step).
c4: the large off-axis collision (N = 4M split 2:1, quadrupole gravity,
    ~64 neighbours): seconds per step and pair interactions per second of
    FP32C and of FP64 graph-captured steps.
Prints one JSON object.
"""
import argparse
import json
import time

import numpy as np

from . import functors, ic
from .system import ParticleSystem, state_from_ic

FIELDS = ("pos", "vel", "dens", "uene", "acc")


def rel_stats(a, b, floor=1e-3):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.ndim > 1:
        d = np.linalg.norm(a - b, axis=-1)
        s = np.linalg.norm(b, axis=-1)
    else:
        d = np.abs(a - b)
        s = np.abs(b)
    r = d / np.maximum(s, floor * s.max())
    return {"median": float(np.median(r)), "p99": float(np.quantile(r, 0.99)), "max": float(r.max())}


def run_steps(state, eta, precision, steps, quadrupole=0, timing_steps=0):
    with functors.Context(precision=precision, eta=eta) as ctx:
        ps = ParticleSystem(ctx, len(state["mass"]), quadrupole=quadrupole)
        ps.upload(state)
        ps.compute_forces()
        e0 = ps.stats()["e_tot"]
        out = {}
        if timing_steps:
            import torch
            ps.step(2)                       # capture and warm the graph
            torch.cuda.synchronize()
            t0 = time.time()
            ps.step(timing_steps)
            torch.cuda.synchronize()
            dt = (time.time() - t0) / timing_steps
            st = ps.stats()
            pairs = st["pairs_density"] + st["pairs_hydro"] + st["pairs_gravity"]
            out.update({"s_per_step": dt, "pairs_per_step": pairs, "interactions_per_s": pairs / dt,
                        "density_walks": st["density_iterations"]})
        else:
            ps.step(steps)
            st = ps.stats()
            out["fields"] = {k: ps.download(k) for k in FIELDS}
            out.update({"e_tot_0": e0, "e_tot": st["e_tot"], "time": st["time"], "steps": st["steps"]})
        ps.close()
    return out


def config1(scale, steps):
    s, eta = ic.config_system("c1", scale=scale)
    s = state_from_ic(s)
    runs = {p: run_steps(s, eta, p, steps) for p in ("fp32c", "fp64")}
    res = {"config": "c1", "n": len(s["mass"]), "steps": steps,
           "time_simulated": runs["fp64"]["time"],
           "fp32c_vs_fp64": {k: rel_stats(runs["fp32c"]["fields"][k], runs["fp64"]["fields"][k]) for k in FIELDS}}
    for p, r in runs.items():
        drift = (r["e_tot"] - r["e_tot_0"]) / abs(r["e_tot_0"])
        res[f"energy_drift_{p}"] = {"total": drift, "per_step": drift / max(r["steps"], 1)}
    return res


def config4(scale, steps):
    s, eta = ic.config_system("c4", scale=scale)
    s = state_from_ic(s)
    res = {"config": "c4", "n": len(s["mass"]), "quadrupole": True}
    for p in ("fp32c", "fp64"):
        res[p] = run_steps(s, eta, p, 0, quadrupole=1, timing_steps=steps)
    res["fp64_over_fp32c"] = res["fp64"]["s_per_step"] / res["fp32c"]["s_per_step"]
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("config", choices=("c1", "c4"))
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--steps", type=int, default=None)
    args = ap.parse_args()
    import torch
    torch.cuda.init()
    if args.config == "c1":
        out = config1(args.scale, args.steps or 200)
    else:
        out = config4(args.scale, args.steps or 5)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
