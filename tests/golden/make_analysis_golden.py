"""Golden vectors of the reference's analysis scripts.

Runs the reference's own Python functions (imported from the reference tree
by path; matplotlib and the plotting helper are replaced by empty modules,
they are only used for figures) on a seeded synthetic two-star state and
stores inputs and outputs in analysis_n2000.npz:

  analysis/common.py            calc_center_of_gravity
  analysis/unbound_mass/unbound_mass.py   calc_unbound_mass
  analysis/lagrange_radius/lagrange_radius.py  calc_r_cg, calc_lagrange_radius
  energy_check/energy_check.py  calc_energy, check_energy_error

Usage (needs the reference tree): python tests/golden/make_analysis_golden.py <reference root>
"""
import importlib.util
import operator
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load(path, name, extra_path):
    sys.path.insert(0, extra_path)
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    sys.path.pop(0)
    return mod


def synthetic(n_half=1000, seed=11):
    """Two clumps with bound and unbound particles (arbitrary consistent units)."""
    rng = np.random.default_rng(seed)
    out = {}
    parts = []
    for s, (c, v, m) in enumerate((((-3.0, 0.2, 0.0), (0.5, -0.1, 0.0), 1.0), ((2.5, -0.3, 0.1), (-0.6, 0.2, 0.0), 0.4))):
        r = np.abs(rng.normal(size=n_half)) ** 1.5
        d = rng.normal(size=(n_half, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        pos = np.array(c) + d * r[:, None]
        vel = np.array(v) + rng.normal(size=(n_half, 3)) * 0.3 * (1 + r[:, None])
        dens = np.exp(-r) * (1 + 0.1 * rng.random(n_half))
        parts.append(dict(pos=pos, vel=vel, mass=np.full(n_half, m / n_half), dens=dens,
                          pot=-m / np.sqrt(r * r + 0.3), uene=0.05 * np.exp(-r) * (1 + rng.random(n_half)),
                          istar=np.full(n_half, s)))
    for k in parts[0]:
        out[k] = np.concatenate([p[k] for p in parts])
    out["id"] = np.arange(2 * n_half)
    return out


def main(ref):
    stub = types.ModuleType("matplotlib")
    stub.pyplot = types.ModuleType("matplotlib.pyplot")
    stub.rcParams = {}
    sys.modules["matplotlib"] = stub
    sys.modules["matplotlib.pyplot"] = stub.pyplot
    plot = types.ModuleType("plot")
    plot.visualization = lambda *a, **k: None
    sys.modules["plot"] = plot

    ana = os.path.join(ref, "analysis")
    common = load(os.path.join(ana, "common.py"), "ref_common", ana)
    unb = load(os.path.join(ana, "unbound_mass", "unbound_mass.py"), "ref_unbound", ana)
    lag = load(os.path.join(ana, "lagrange_radius", "lagrange_radius.py"), "ref_lagrange", ana)
    ec_dir = os.path.join(ref, "energy_check")
    ene = load(os.path.join(ec_dir, "energy_check.py"), "ref_energy", ec_dir)

    s = synthetic()
    n = len(s["mass"])

    def particles(idx, mod):
        ps = [mod.Particle() for _ in idx]
        for p, i in zip(ps, idx):
            p.p_id = float(s["id"][i])
            p.istar = float(s["istar"][i])
            p.mass = float(s["mass"][i])
            p.pos = s["pos"][i].astype(float).copy()
            p.vel = s["vel"][i].astype(float).copy()
            p.dens = float(s["dens"][i])
            p.pot = float(s["pot"][i])
            p.uene = float(s["uene"][i])
        return ps

    gold = {k: v for k, v in s.items()}
    for name, idx in (("all", np.arange(n)), ("star0", np.arange(n // 2)), ("star1", np.arange(n // 2, n))):
        p = particles(idx, common)
        pc, vc = common.calc_center_of_gravity(p)
        gold[f"cg_{name}"] = np.concatenate([pc, vc])
        total = sum(q.mass for q in p)
        b, u = unb.calc_unbound_mass(p, total, vc)
        gold[f"bound_{name}"] = np.array([b, u])
        # Lagrange radii about the density-weighted centre
        pl = particles(idx, lag)
        pcg = lag.calc_center_of_gravity(pl) if hasattr(lag, "calc_center_of_gravity") else pc
        pcg = pcg[0] if isinstance(pcg, tuple) else pcg
        for q in pl:
            lag.calc_r_cg(q, pcg)
        pl.sort(key=operator.attrgetter("r_cg"))
        lr = [[] for _ in range(9)]
        lag.calc_lagrange_radius(pl, lr, sum(q.mass for q in pl), len(pl))
        gold[f"lagrange_{name}"] = np.array([v[0] for v in lr if v])
        gold[f"lagrange_centre_{name}"] = np.asarray(pcg, dtype=float)
    # two-star orbital energy (stars split by halves, radii R1 = R2 = 2.0)
    ene.R1 = 2.0
    ene.R2 = 2.0
    gold["orbit_energy"] = np.array([ene.calc_energy(particles(np.arange(n), ene))])
    gold["orbit_G"] = np.array([ene.G])
    gold["orbit_R"] = np.array([2.0, 2.0])
    # energy error of a time series (time, energy)
    t = np.arange(0, 50.0, 1.0)
    e = -1.0 + 1e-4 * np.sin(t / 3.0) + 2e-5 * t / 50.0
    ts = np.stack([t, e], axis=1)
    gold["energy_series"] = ts
    gold["energy_error"] = np.array(ene.check_energy_error(ts, 40.0), dtype=float)
    np.savez_compressed(os.path.join(HERE, "analysis_n2000.npz"), **gold)
    print("wrote", os.path.join(HERE, "analysis_n2000.npz"), {k: v.shape for k, v in gold.items()})


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit(f"usage: python {os.path.relpath(__file__)} <reference root>")
    main(sys.argv[1])
