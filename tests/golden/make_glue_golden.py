"""Generates tests/golden/glue_n256.npz: the reference's own per-particle step
glue run on seeded synthetic inputs.

The glue is HelmholtzGas's ideal-gas EOS, time step, energy, predictor and
corrector and alpha derivative, SPH's Balsara switch and sumAcceleration, and
calcKernelSupportRadiusMaximum (sph_yamauchi/run/hdr_hgas.hpp, hdr_sph.hpp,
hdr_util.hpp), compiled from the reference tree by

    make -C oracle ref REF_DIR=<reference root>/sph_yamauchi/run

into oracle/_ref/libsph_ref_glue.so (oracle/ref_glue.cpp).  Inputs and the
reference's outputs are stored together; tests/test_oracle.py replays the
inputs through the C restatement in oracle/sph_oracle.c.

Run from the repository root after building that library:
    python tests/golden/make_glue_golden.py
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402

N = 256
SEED = 20261204
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "glue_n256.npz")
C_DT, DT_MAX, ALPHA_MAX, ALPHA_MIN = 0.1, 10.0, 2.0, 0.1


def inputs(seed=SEED, n=N):
    rng = np.random.default_rng(seed)
    g = {}
    g["mass"] = rng.uniform(5.0, 20.0, n)
    g["pos"] = rng.normal(scale=3000.0, size=(n, 3)) + np.array([2.0e4, -1.0e4, 5.0e3])
    g["vel"] = rng.normal(scale=300.0, size=(n, 3))
    g["acc"] = rng.normal(scale=10.0, size=(n, 3))
    g["dens"] = np.exp(rng.uniform(np.log(1e-3), np.log(1e2), n))
    g["uene"] = np.exp(rng.uniform(np.log(1e3), np.log(1e7), n))
    g["ksr"] = np.exp(rng.uniform(np.log(2.0), np.log(300.0), n))
    dv = rng.normal(scale=0.05, size=n)
    dv[::17] = 0.0                     # no compression: the dt_max branch
    g["divv"] = dv
    g["rotv"] = np.abs(rng.normal(scale=0.05, size=n))
    g["rotv"][::23] = 0.0
    g["alph"] = rng.uniform(0.1, 2.0, n)
    g["alphu"] = np.zeros(n)
    g["udot"] = rng.normal(scale=1e3, size=n)
    g["adot"] = rng.normal(scale=1e-2, size=n)
    g["adotu"] = np.zeros(n)
    g["pot"] = -np.exp(rng.uniform(np.log(1e4), np.log(1e7), n))
    g["accg1"] = rng.normal(scale=0.1, size=(n, 3))
    g["accg2"] = rng.normal(scale=20.0, size=(n, 3))
    g["acch"] = rng.normal(scale=20.0, size=(n, 3))
    g["istar"] = (rng.random(n) < 0.6).astype(np.int32)
    g["dt"] = np.array(2.5)
    return g


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def reference_outputs(g):
    lib = orc.ref_glue_lib()
    n = len(g["mass"])
    f = {k: np.ascontiguousarray(v) for k, v in g.items()}
    o = {}
    o["pres"], o["vsnd"] = np.empty(n), np.empty(n)
    lib.ref_glue_eos(n, _p(f["dens"]), _p(f["uene"]), _p(o["pres"]), _p(o["vsnd"]))
    o["bswt"] = np.empty(n)
    lib.ref_glue_balsara(n, _p(f["divv"]), _p(f["rotv"]), _p(o["vsnd"]), _p(f["ksr"]), _p(o["bswt"]))
    o["adot"] = np.empty(n)
    lib.ref_glue_alpha_dot(n, _p(f["divv"]), _p(f["alph"]), _p(o["vsnd"]), _p(f["ksr"]), ALPHA_MAX, ALPHA_MIN,
                           _p(o["adot"]))
    vsmx = np.ascontiguousarray(2.0 * o["vsnd"] + 3.0 * np.abs(f["divv"]) * f["ksr"])
    o["vsmx_in"] = vsmx
    o["dt_particle"] = np.empty(n)
    lib.ref_glue_timestep(n, _p(f["ksr"]), _p(vsmx), _p(f["divv"]), _p(f["accg1"]), _p(f["accg2"]), C_DT, DT_MAX,
                          _p(o["dt_particle"]))
    o["energy_particle"] = np.empty(n)
    lib.ref_glue_energy(n, _p(f["mass"]), _p(f["vel"]), _p(f["uene"]), _p(f["pot"]), _p(o["energy_particle"]))
    p = {k: f[k].copy() for k in ("pos", "vel", "uene", "alph", "alphu")}
    p["vel2"], p["uene2"], p["alph2"], p["alphu2"] = (np.empty_like(f["vel"]), np.empty(n), np.empty(n),
                                                      np.empty(n))
    dt = float(g["dt"])
    lib.ref_glue_predict(n, dt, _p(p["pos"]), _p(p["vel"]), _p(f["acc"]), _p(p["vel2"]), _p(p["uene"]),
                         _p(p["uene2"]), _p(f["udot"]), _p(p["alph"]), _p(p["alph2"]), _p(f["adot"]),
                         _p(p["alphu"]), _p(p["alphu2"]), _p(f["adotu"]))
    for k, v in p.items():
        o["pred_" + k] = v
    c = {k: np.empty_like(p[k]) for k in ("vel", "uene", "alph", "alphu")}
    acc_new = np.ascontiguousarray(f["acc"][::-1])     # the new derivatives of the corrector
    udot_new = np.ascontiguousarray(f["udot"][::-1])
    adot_new = np.ascontiguousarray(f["adot"][::-1])
    lib.ref_glue_correct(n, dt, _p(c["vel"]), _p(p["vel2"]), _p(acc_new), _p(c["uene"]), _p(p["uene2"]),
                         _p(udot_new), _p(c["alph"]), _p(p["alph2"]), _p(adot_new), _p(c["alphu"]),
                         _p(p["alphu2"]), _p(f["adotu"]))
    for k, v in c.items():
        o["corr_" + k] = v
    o["acc_sum"] = np.empty_like(f["acch"])
    lib.ref_glue_sum_acceleration(n, _p(f["acch"]), _p(f["accg1"]), _p(f["accg2"]), _p(o["acc_sum"]))
    o["ksrmax"] = np.array(lib.ref_glue_ksrmax(n, _p(f["mass"]), _p(f["pos"]), _p(f["vel"]), _p(f["istar"]),
                                               _p(f["dens"])))
    return o


def main():
    if not orc.ref_glue_available():
        sys.exit("oracle/_ref/libsph_ref_glue.so is missing: make -C oracle ref REF_DIR=<reference>/sph_yamauchi/run")
    g = inputs()
    o = reference_outputs(g)
    np.savez_compressed(OUT, **{"in_" + k: v for k, v in g.items()}, **{"ref_" + k: v for k, v in o.items()},
                        c_dt=C_DT, dt_max=DT_MAX, alpha_max=ALPHA_MAX, alpha_min=ALPHA_MIN)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
