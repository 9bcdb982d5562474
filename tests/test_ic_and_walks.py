"""CPU tests of the initial conditions (polytropes, two-star placement, the
benchmark configurations) and of the host-built walks that feed the oracle
and the reference arm of the benchmark."""
import math

import numpy as np

from research_codes_gb300 import ic, units, walks


def test_polytrope_mass_radius_and_profile():
    s = ic.polytrope(4000, 1.0, 1.0, 1.5, seed=2)
    M = units.SOLAR_MASS / units.UNIT_MASS
    R = units.SOLAR_RADIUS / units.UNIT_LENGTH
    assert abs(s["mass"].sum() - M) < 1e-12 * M
    r = np.linalg.norm(s["pos"], axis=1)
    assert r.max() <= R * (1 + 1e-9)
    # half of the mass inside the Lane-Emden half-mass radius: the particles
    # are placed by enclosed mass, so the median radius is that radius
    xi, th, dth = ic.lane_emden(1.5)
    mfrac = (xi * xi * dth) / (xi[-1] ** 2 * dth[-1])
    r_half = np.interp(0.5, mfrac, xi) / xi[-1] * R
    assert abs(np.median(r) - r_half) < 0.02 * R
    # density falls outwards, and uene = n P / rho with P = K rho^(1+1/n)
    o = np.argsort(r)
    assert s["dens"][o[0]] > s["dens"][o[-1]]
    assert np.allclose(s["uene"], 1.5 * s["K"] * s["dens"] ** (1.0 / 1.5), rtol=1e-12)
    assert (s["vel"] == 0).all()


def test_two_stars_centre_of_mass_frame():
    a = ic.polytrope(500, 10.0, 4.0, 3.0, seed=1)
    b = ic.polytrope(300, 3.0, 1.5, 1.5, seed=2)
    sep, imp = 1.5e4, 2.0e3
    v = ic.escape_speed(a["M"] + b["M"], math.hypot(sep, imp))
    s = ic.two_stars(a, b, sep, imp, v)
    m = s["mass"]
    com = (m[:, None] * s["pos"]).sum(0) / m.sum()
    mom = (m[:, None] * s["vel"]).sum(0)
    # stars are placed by their centres; each star's particle sample sits
    # within a small fraction of its radius of that centre
    assert np.abs(com).max() < 0.01 * a["R"]
    assert np.abs(mom).max() < 1e-9 * m.sum() * v
    c1 = s["pos"][s["istar"] == 0].mean(0)
    c2 = s["pos"][s["istar"] == 1].mean(0)
    assert np.allclose(c2 - c1, [sep, imp, 0.0], rtol=0, atol=0.05 * sep)
    dv = s["vel"][s["istar"] == 1][0] - s["vel"][s["istar"] == 0][0]
    assert np.allclose(dv, [-v, 0.0, 0.0], rtol=1e-12)
    assert abs(v - math.sqrt(2 * units.G * (a["M"] + b["M"]) / math.hypot(sep, imp))) < 1e-12 * v


def test_benchmark_configurations_at_small_scale():
    for name, n_full in (("c0", 10_000), ("c1", 200_000), ("c2", 1_000_000), ("c3", 100_000), ("c4", 4_000_000)):
        s, eta = ic.config_system(name, scale=0.01)
        n = len(s["mass"])
        assert abs(n - 0.01 * n_full) <= 2, (name, n)
        assert eta in (1.18, 1.28)
        assert s["pos"].shape == (n, 3) and (s["ksr"] > 0).all() and (s["uene"] > 0).all()


def test_gather_and_symmetric_lists_are_complete():
    rng = np.random.default_rng(4)
    pos = rng.uniform(-1.0, 1.0, size=(600, 3))
    h = rng.uniform(0.05, 0.25, size=600)
    groups = walks.make_groups(pos, 32)
    assert sorted(np.concatenate(groups).tolist()) == list(range(600))
    gl = walks.gather_lists(pos, h, groups)
    sl = walks.symmetric_lists(pos, h, groups)
    for g, lg, ls in zip(groups, gl, sl):
        have_g, have_s = set(lg.tolist()), set(ls.tolist())
        for i in g:
            d = np.linalg.norm(pos - pos[i], axis=1)
            assert set(np.nonzero(d < h[i])[0].tolist()) <= have_g
            assert set(np.nonzero(d < np.maximum(h[i], h))[0].tolist()) <= have_s


def test_host_gravity_lists_reproduce_direct_summation():
    """Near particles plus far-cell monopoles (the reference arm's gravity
    lists) against direct summation, both through the oracle's functors."""
    from oracle import oracle as orc
    from research_codes_gb300 import abi
    s = ic.polytrope(20000, 1.0, 1.0, 1.5, seed=6)
    n = len(s["mass"])
    state = dict(pos=s["pos"], mass=s["mass"], ksr=s["ksr"])
    eps2 = (s["ksr"] / units.KSRH) ** 2
    groups = walks.make_groups(s["pos"], 64)
    el, sl = walks.gravity_lists(s["pos"], s["mass"], eps2, groups)
    allj = walks.gravity_epj(np.arange(n), state)
    errs, entries, n_spj, picked = [], 0, 0, 0
    for g, e, spj in list(zip(groups, el, sl))[::40]:
        epi = walks.gravity_epi(g, state)
        tree = orc.gravity(epi, walks.gravity_epj(e, state), spj)
        direct = orc.gravity(epi, allj)
        errs.append(np.linalg.norm(tree["acc"] - direct["acc"], axis=1) / np.linalg.norm(direct["acc"], axis=1))
        entries += len(e) + len(spj)
        n_spj += len(spj)
        picked += 1
    # monopoles stand in for far particles: the lists are shorter overall
    assert n_spj > 0 and entries < 0.9 * picked * n
    errs = np.concatenate(errs)
    assert np.median(errs) < 5e-3 and errs.max() < 5e-2, (np.median(errs), errs.max())
