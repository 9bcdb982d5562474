"""Analysis of the state (the reference's post-processing scripts): the
oracle restatement against the reference's own functions (golden vectors),
and the device implementation against both."""
import os

import numpy as np
import pytest

from conftest import ROOT
from oracle import analysis_oracle as ao
from research_codes_gb300 import analysis

GOLD = os.path.join(ROOT, "tests", "golden", "analysis_n2000.npz")
SETS = (("all", None), ("star0", 0), ("star1", 1))


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def _sel(g, star):
    return np.ones(len(g["mass"]), bool) if star is None else g["istar"] == star


def test_oracle_matches_reference_scripts(gold):
    g = gold
    for name, star in SETS:
        s = _sel(g, star)
        pc, vc = ao.centre_of_gravity(g["pos"][s], g["vel"][s], g["dens"][s])
        assert np.allclose(np.concatenate([pc, vc]), g[f"cg_{name}"], rtol=1e-13, atol=1e-15)
        b, u = ao.bound_mass(g["vel"][s], g["pot"][s], g["uene"][s], g["mass"][s], vc)
        assert np.allclose([b, u], g[f"bound_{name}"], rtol=1e-12)
        lr = ao.lagrange_radii(g["pos"][s], g["mass"][s], g[f"lagrange_centre_{name}"])
        assert np.allclose(lr, g[f"lagrange_{name}"], rtol=1e-13)
    e = ao.orbit_energy(g["pos"], g["vel"], g["dens"], g["mass"], g["istar"], *g["orbit_R"], g["orbit_G"][0])
    assert np.isclose(e, g["orbit_energy"][0], rtol=1e-12)
    assert np.allclose(ao.energy_error(g["energy_series"], 40.0), g["energy_error"], rtol=1e-13)
    ts = g["energy_series"]
    assert np.allclose(analysis.energy_error(ts[:, 0], ts[:, 1], 40.0), g["energy_error"], rtol=1e-13)
    assert np.allclose(analysis.lagrange_from_sorted(*_sorted(g, None)), g["lagrange_all"], rtol=1e-13)


def _sorted(g, star):
    s = _sel(g, star)
    d = g["pos"][s] - g["lagrange_centre_all"]
    r = np.sqrt(np.sum(d * d, axis=1))
    o = np.argsort(r, kind="stable")
    return r[o], g["mass"][s][o]


@pytest.mark.gpu
def test_device_analysis_matches_reference(gold):
    from research_codes_gb300 import functors
    from research_codes_gb300.system import ParticleSystem
    g = gold
    n = len(g["mass"])
    with functors.Context() as ctx:
        ps = ParticleSystem(ctx, n, n_group=64)
        ps.upload({"id": g["id"], "istar": g["istar"], "mass": g["mass"], "pos": g["pos"], "vel": g["vel"],
                   "uene": g["uene"], "ksr": np.ones(n)})
        ps.set_field("dens", g["dens"])
        ps.set_field("pot", g["pot"])
        for name, star in SETS:
            pc, vc = analysis.centre_of_gravity(ps, star)
            assert np.allclose(np.concatenate([pc, vc]), g[f"cg_{name}"], rtol=1e-12, atol=1e-14), name
            assert np.allclose(analysis.bound_mass(ps, star, vc), g[f"bound_{name}"], rtol=1e-12), name
            lr = analysis.lagrange_radii(ps, star, center=g[f"lagrange_centre_{name}"])
            assert np.allclose(lr, g[f"lagrange_{name}"], rtol=1e-12), name
            assert np.allclose(analysis.lagrange_radii(ps, star), g[f"lagrange_{name}"], rtol=1e-9), name
        e = analysis.binary_orbit_energy(ps, *g["orbit_R"], g["orbit_G"][0])
        assert np.isclose(e, g["orbit_energy"][0], rtol=1e-11)
        ps.close()
