"""Generates the golden vectors in this directory from the reference's own
functors.

The reference (yamauchi1132/Research_Codes) ships no known-answer tests for
the SPH interaction path, so the golden outputs are produced by running its
own scalar FP64 CPU functors (calcDensity, calcHydro, calcGravity<EPJ/SPJ>),
compiled from the reference source tree by `make -C oracle ref` (the library
oracle/_ref/libsph_ref.so, see oracle/ref_bridge.cpp), on seeded synthetic
inputs: a small n=1.5 polytrope from research_codes_gb300.ic with a
rotating, expanding velocity field.  The inputs and the reference outputs are
stored together; the tests replay the inputs through the oracle restatement
and through the CUDA engine.

Run from the repository root:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from research_codes_gb300 import abi, ic, units, walks  # noqa: E402

SEED = 20261203
N = 1000
N_GROUP = 64
KEEP = [0, 7, 15]          # walks stored per interaction kind
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "functors_n1000.npz")


def system(seed=SEED, n=N):
    rng = np.random.default_rng(seed)
    s = ic.polytrope(n, 1.0, 1.0, 1.5, seed=seed, eta=units.ETA_REFERENCE)
    pos = s["pos"]
    R = s["R"]
    omega = np.array([0.3, -0.2, 1.0]) * 2e-3
    vel = np.cross(omega, pos) + 1e-3 * pos + rng.normal(scale=0.05, size=pos.shape)
    s["vel"] = vel
    s["id"] = np.arange(n, dtype=np.int64) + 7          # ids need not equal indices
    s["ksr"] = s["ksr"] * rng.uniform(0.9, 1.1, size=n)  # imperfect first guess
    s["rs"] = 1.1 * s["ksr"]                             # hdr_density.hpp:376-379
    s["R"] = R
    return s, rng


def _subset(prefix, items, keep, out, i_off):
    sel = [items[k] for k in keep]
    epi, epj, io, jo = walks.concat_walks(sel)
    o = np.concatenate([out[i_off[k]:i_off[k + 1]] for k in keep])
    return {f"{prefix}_epi": epi, f"{prefix}_epj": epj, f"{prefix}_i_off": io,
            f"{prefix}_j_off": jo, f"{prefix}_out": o}


def main():
    if not orc.ref_available():
        orc.build(ref=True)
    s, rng = system()
    pos = s["pos"]
    groups = walks.make_groups(pos, N_GROUP)
    data = {"meta": np.array(f"seed={SEED} n={N} n_group={N_GROUP} eta=1.6 "
                             "generator=tests/golden/make_golden.py impl=ref")}

    # --- density: all groups (so every particle gets a result for hydro inputs)
    jl = walks.gather_lists(pos, s["rs"], groups)
    items = [(walks.density_epi(g, s), walks.density_epj(j, s)) for g, j in zip(groups, jl)]
    # edge cases: a single i-particle; a self-only j-list
    g0 = groups[3][:1]
    items.append((walks.density_epi(g0, s), walks.density_epj(jl[3], s)))
    items.append((walks.density_epi(g0, s), walks.density_epj(g0, s)))
    epi, epj, i_off, j_off = walks.concat_walks(items)
    out = np.zeros(len(epi), abi.Density)
    for w in range(len(items)):
        a, b = slice(i_off[w], i_off[w + 1]), slice(j_off[w], j_off[w + 1])
        out[a] = orc.density(epi[a], epj[b], eta=1.6, ksr_max=0.0, impl="ref")
    keep = KEEP + [len(groups), len(groups) + 1]
    data.update(_subset("dens", items, keep, out, i_off))

    # --- density with an active ksrmax clamp (hdr_density.hpp:291-292)
    kmax = float(np.median(s["ksr"]) * 0.9)
    sub = [items[k] for k in KEEP[:3]]
    epi_c, epj_c, io_c, jo_c = walks.concat_walks(sub)
    out_c = np.zeros(len(epi_c), abi.Density)
    for w in range(len(sub)):
        a, b = slice(io_c[w], io_c[w + 1]), slice(jo_c[w], jo_c[w + 1])
        out_c[a] = orc.density(epi_c[a], epj_c[b], eta=1.6, ksr_max=kmax, impl="ref")
    data.update(densc_epi=epi_c, densc_epj=epj_c, densc_i_off=io_c, densc_j_off=jo_c,
                densc_out=out_c, densc_ksr_max=np.array(kmax))

    # --- per-particle state for the hydro inputs (assemble from the density run)
    n = len(pos)
    dres = np.zeros(n, abi.Density)
    for w, g in enumerate(groups):
        dres[g] = out[i_off[w]:i_off[w + 1]]
    s["dens"] = dres["dens"]
    s["grdh"] = dres["grdh"]
    s["ksr"] = dres["ksr"]
    pres, vsnd = orc.eos(s["dens"], s["uene"])
    s["pres"], s["vsnd"] = pres, vsnd
    s["bswt"] = orc.balsara(dres["divv"], dres["rotv"], vsnd, s["ksr"])
    s["alph"] = rng.uniform(0.1, 2.0, n)
    s["alphu"] = rng.uniform(0.0, 1.0, n)
    s["uene"] = s["uene"] * rng.uniform(0.8, 1.2, n)
    s["eta"] = rng.uniform(0.0, 0.3, n)

    hl = walks.symmetric_lists(pos, s["ksr"], groups)
    hitems = [(walks.hydro_epi(g, s), walks.hydro_epj(j, s)) for g, j in zip(groups, hl)]
    hitems.append((walks.hydro_epi(g0, s), walks.hydro_epj(g0, s)))   # self only
    keep = KEEP + [len(groups)]
    hitems = [hitems[k] for k in keep]
    epi, epj, i_off, j_off = walks.concat_walks(hitems)
    out = np.zeros(len(epi), abi.Hydro)
    for w in range(len(hitems)):
        a, b = slice(i_off[w], i_off[w + 1]), slice(j_off[w], j_off[w + 1])
        out[a] = orc.hydro(epi[a], epj[b], impl="ref")
    data.update(hydro_epi=epi, hydro_epj=epj, hydro_i_off=i_off, hydro_j_off=j_off,
                hydro_out=out)

    # --- gravity: EPJ near the group + SPJ monopoles of far cells
    eps2 = (s["ksr"] / units.KSRH) ** 2
    el, sl = walks.gravity_lists(pos, s["mass"], eps2, groups, near_factor=0.6, cell_frac=0.1)
    gi, gj, gs = [], [], []
    for k in KEEP:
        g, e, sp = groups[k], el[k], sl[k]
        gi.append(walks.gravity_epi(g, s))
        gj.append(walks.gravity_epj(e, s))
        gs.append(sp)
    i_off = np.concatenate([[0], np.cumsum([len(a) for a in gi])]).astype(np.int64)
    j_off = np.concatenate([[0], np.cumsum([len(a) for a in gj])]).astype(np.int64)
    s_off = np.concatenate([[0], np.cumsum([len(a) for a in gs])]).astype(np.int64)
    epi, epj, spj = np.concatenate(gi), np.concatenate(gj), np.concatenate(gs)
    out = np.zeros(len(epi), abi.Gravity)
    for w in range(len(gi)):
        a = slice(i_off[w], i_off[w + 1])
        out[a] = orc.gravity(epi[a], epj[j_off[w]:j_off[w + 1]], spj[s_off[w]:s_off[w + 1]],
                             impl="ref")
    data.update(grav_epi=epi, grav_epj=epj, grav_spj=spj, grav_i_off=i_off, grav_j_off=j_off,
                grav_s_off=s_off, grav_out=out)

    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
