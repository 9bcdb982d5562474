"""CPU check of the double-float hydro pair formula of the FP32C engine.

csrc/hydro_df.cuh and csrc/df32.cuh compile for the host as plain C++
(without FP contraction), with the packed two-lane type emulated per half.
tests/hydro_df_host.cpp builds the per-particle records as
make_hydro_records does and sums every pair of a walk (self pair excluded);
this test compiles it with g++ and compares the results with the
reference's own outputs (tests/golden/functors_n1000.npz): within 1e-5 per
particle for acch, accg and du/dt, 1e-4 for diffu, with the floors of the
GPU tests; the packed order must give the same sums as the one-pair order
to double-float rounding.  The device differs only in its 1/sqrt seed
(refined by the same Newton step).
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import rel_err, walk_slices

HERE = os.path.dirname(os.path.abspath(__file__))


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "vector_types.h")):
            return os.path.join(d, "include")
    return None


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    inc = _cuda_include()
    if shutil.which("g++") is None or inc is None:
        pytest.skip("g++ or the CUDA headers are missing")
    so = str(tmp_path_factory.mktemp("dfh") / "libhydro_df_host.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", f"-I{inc}", "-o", so,
                    os.path.join(HERE, "hydro_df_host.cpp")], check=True)
    return ctypes.CDLL(so)


def _records(e, mass):
    r = np.zeros((len(e), 17))
    r[:, 0:3] = e["pos"]
    r[:, 3:6] = e["vel"]
    r[:, 6] = mass
    for k, f in enumerate(("hinv", "pres", "presc", "bswt", "dens", "vsnd", "alph", "alphu", "thrm", "eta")):
        r[:, 7 + k] = e[f]
    return np.ascontiguousarray(r)


def _walk(lib, epi, epj, packed):
    P = ctypes.c_void_p
    ri, rj = _records(epi, 0.0), _records(epj, epj["mass"])
    idi = np.ascontiguousarray(epi["id"], np.int64)
    idj = np.ascontiguousarray(epj["id"], np.int64)
    out = np.zeros((len(epi), 8))
    lib.df_walk(len(epi), ri.ctypes.data_as(P), idi.ctypes.data_as(P), len(epj), rj.ctypes.data_as(P),
                idj.ctypes.data_as(P), int(packed), out.ctypes.data_as(P))
    return out


def test_double_float_hydro_matches_reference_golden(lib):
    g = np.load(os.path.join(HERE, "golden", "functors_n1000.npz"))
    worst = {"acch": 0.0, "accg": 0.0, "udot": 0.0, "diffu": 0.0}
    for _, a, b in walk_slices(g["hydro_i_off"], g["hydro_j_off"]):
        epi, epj = g["hydro_epi"][a], g["hydro_epj"][b]
        one = _walk(lib, epi, epj, False)
        two = _walk(lib, epi, epj, True)
        # the two orders differ only in the grouping of double-float sums
        assert np.allclose(one, two, rtol=1e-11, atol=1e-11 * np.abs(one).max())
        ref = g["hydro_out"][a]
        worst["acch"] = max(worst["acch"], rel_err(two[:, 0:3], ref["acch"], floor_frac=1e-3).max())
        worst["accg"] = max(worst["accg"], rel_err(two[:, 3:6], ref["accg"], floor_frac=1e-3).max())
        worst["udot"] = max(worst["udot"], rel_err(two[:, 6], ref["udot"], floor_frac=1e-3).max())
        worst["diffu"] = max(worst["diffu"], rel_err(two[:, 7], ref["diffu"], floor_frac=1e-2).max())
    assert worst["acch"] < 1e-5 and worst["accg"] < 1e-5 and worst["udot"] < 1e-5, worst
    assert worst["diffu"] < 1e-4, worst


def test_double_float_hydro_far_from_origin_vs_oracle(lib):
    """Two blobs 3e4 from the origin colliding at +-400: separations and
    velocity differences live mostly in the records' lo parts."""
    from oracle import oracle as orc
    from research_codes_gb300 import walks
    rng = np.random.default_rng(13)
    n = 3000
    a = rng.normal(size=(n // 2, 3))
    b = rng.normal(size=(n - n // 2, 3)) * 0.7 + np.array([2.5, 0.4, 0.0])
    pos = np.concatenate([a, b]) + 3.0e4
    vel = np.concatenate([np.tile([400.0, 0, 0], (n // 2, 1)), np.tile([-400.0, 0, 0], (n - n // 2, 1))])
    vel += rng.normal(scale=1.0, size=vel.shape)
    mass = rng.uniform(0.8, 1.2, n) / n
    rho = np.exp(-0.5 * (np.linalg.norm(pos - pos.mean(0), axis=1) ** 2)) + 0.05
    h = 1.2 * 1.936492 * (mass / rho) ** (1 / 3) * 0.25
    s = dict(pos=pos, vel=vel, mass=mass, ksr=h, id=rng.permutation(n).astype(np.int64),
             pres=rng.uniform(1, 2, n) * 1e-3, grdh=rng.uniform(0.8, 1.2, n), dens=rng.uniform(1, 3, n),
             bswt=rng.uniform(0, 1, n), vsnd=rng.uniform(1, 2, n) * 50, alph=rng.uniform(0.1, 2, n),
             alphu=rng.uniform(0, 1, n), uene=rng.uniform(1, 2, n) * 1e3, eta=rng.uniform(0, 0.3, n))
    groups = walks.make_groups(s["pos"], 64)
    lists = walks.symmetric_lists(s["pos"], s["ksr"], groups)
    outs, refs = [], []
    for g, j in list(zip(groups, lists))[::5]:
        epi, epj = walks.hydro_epi(g, s), walks.hydro_epj(j, s)
        outs.append(_walk(lib, epi, epj, True))
        refs.append(orc.hydro(epi, epj))
    o, r = np.concatenate(outs), np.concatenate(refs)
    assert rel_err(o[:, 0:3], r["acch"], floor_frac=1e-3).max() < 1e-5
    assert rel_err(o[:, 3:6], r["accg"], floor_frac=1e-3).max() < 1e-5
    assert rel_err(o[:, 6], r["udot"], floor_frac=1e-3).max() < 1e-5
