"""The oracle restatement (oracle/sph_oracle.c) against the reference's own
functors: first the committed golden vectors, then (where the reference tree
is present and oracle/_ref builds) fresh seeded cases run through both."""
import numpy as np
import pytest

from conftest import rel_err, walk_slices
from oracle import oracle as orc
from research_codes_gb300 import abi, walks

TOL = 1e-10   # FP64 vs FP64, differing only in operation order


def _check_density(out, ref, tol=TOL):
    for f in ("dens", "divv", "rotv", "grdh", "ksr"):
        assert rel_err(out[f], ref[f]).max() < tol, f
    assert np.array_equal(out["np"], ref["np"])
    assert np.array_equal(out["itr"], ref["itr"])


def test_density_golden(golden):
    g = golden
    for _, a, b in walk_slices(g["dens_i_off"], g["dens_j_off"]):
        out = orc.density(g["dens_epi"][a], g["dens_epj"][b], eta=1.6, ksr_max=0.0)
        _check_density(out, g["dens_out"][a])


def test_density_clamp_golden(golden):
    g = golden
    kmax = float(g["densc_ksr_max"])
    n_clamped = 0
    for _, a, b in walk_slices(g["densc_i_off"], g["densc_j_off"]):
        out = orc.density(g["densc_epi"][a], g["densc_epj"][b], eta=1.6, ksr_max=kmax)
        _check_density(out, g["densc_out"][a])
        n_clamped += int((out["ksr"] == kmax).sum())
    assert n_clamped > 0


def test_density_self_only_golden(golden):
    """The last stored density walk has a j-list holding only the i-particle."""
    g = golden
    io, jo = g["dens_i_off"], g["dens_j_off"]
    w = len(io) - 2
    assert io[w + 1] - io[w] == 1 and jo[w + 1] - jo[w] == 1
    ref = g["dens_out"][io[w]:io[w + 1]]
    out = orc.density(g["dens_epi"][io[w]:io[w + 1]], g["dens_epj"][jo[w]:jo[w + 1]])
    _check_density(out, ref)
    assert ref["np"][0] == 1


def test_hydro_golden(golden):
    g = golden
    for _, a, b in walk_slices(g["hydro_i_off"], g["hydro_j_off"]):
        out = orc.hydro(g["hydro_epi"][a], g["hydro_epj"][b])
        ref = g["hydro_out"][a]
        for f in ("acch", "accg", "udot", "vsmx", "diffu"):
            assert rel_err(out[f], ref[f]).max() < TOL, f


def test_gravity_golden(golden):
    g = golden
    io, jo, so = g["grav_i_off"], g["grav_j_off"], g["grav_s_off"]
    for w in range(len(io) - 1):
        a = slice(io[w], io[w + 1])
        out = orc.gravity(g["grav_epi"][a], g["grav_epj"][jo[w]:jo[w + 1]],
                          g["grav_spj"][so[w]:so[w + 1]])
        ref = g["grav_out"][a]
        for f in ("acc", "pot", "eta"):
            assert rel_err(out[f], ref[f]).max() < TOL, f


def test_gravity_accumulates(golden):
    """calcGravity adds into the force (hdr_gravity.hpp:333-337)."""
    g = golden
    a = slice(0, int(g["grav_i_off"][1]))
    b = slice(0, int(g["grav_j_off"][1]))
    once = orc.gravity(g["grav_epi"][a], g["grav_epj"][b])
    twice = orc.gravity(g["grav_epi"][a], g["grav_epj"][b], out=once.copy())
    assert rel_err(twice["pot"], 2 * once["pot"]).max() < 1e-14


def test_walk_batched_matches_single(golden):
    g = golden
    out, nt = orc.density_walks(g["dens_i_off"], g["dens_j_off"], g["dens_epi"],
                                g["dens_epj"], nthreads=2)
    assert nt >= 1
    _check_density(out, g["dens_out"])
    hout, _ = orc.hydro_walks(g["hydro_i_off"], g["hydro_j_off"], g["hydro_epi"],
                              g["hydro_epj"], nthreads=2)
    assert rel_err(hout["acch"], g["hydro_out"]["acch"]).max() < TOL


# ---- live comparison with the reference build (only where it exists) -------

needs_ref = pytest.mark.skipif(not orc.ref_available(), reason="oracle/_ref not built here")


def _random_system(seed, n=600):
    rng = np.random.default_rng(seed)
    pos = rng.normal(size=(n, 3)) * np.array([1.0, 0.7, 1.3])
    vel = rng.normal(size=(n, 3)) + 0.3 * np.cross([0.0, 0.0, 1.0], pos)
    mass = rng.uniform(0.5, 1.5, n)
    h = rng.uniform(0.3, 0.6, n)
    s = dict(pos=pos, vel=vel, mass=mass, ksr=h, rs=1.1 * h,
             id=np.arange(n, dtype=np.int64) * 3 + 1)
    return s, rng


@needs_ref
@pytest.mark.parametrize("seed", [1, 2])
def test_density_vs_reference_live(seed):
    s, _ = _random_system(seed)
    groups = walks.make_groups(s["pos"], 48)
    jl = walks.gather_lists(s["pos"], s["rs"], groups)
    for g, j in list(zip(groups, jl))[::3]:
        epi, epj = walks.density_epi(g, s), walks.density_epj(j, s)
        _check_density(orc.density(epi, epj), orc.density(epi, epj, impl="ref"))


@needs_ref
def test_hydro_gravity_vs_reference_live():
    s, rng = _random_system(3)
    n = len(s["mass"])
    s.update(pres=rng.uniform(1, 2, n), grdh=rng.uniform(0.8, 1.2, n), dens=rng.uniform(1, 3, n),
             bswt=rng.uniform(0, 1, n), vsnd=rng.uniform(1, 2, n), alph=rng.uniform(0.1, 2, n),
             alphu=rng.uniform(0, 1, n), uene=rng.uniform(1, 2, n), eta=rng.uniform(0, 0.3, n))
    groups = walks.make_groups(s["pos"], 48)
    hl = walks.symmetric_lists(s["pos"], s["ksr"], groups)
    for g, j in list(zip(groups, hl))[::4]:
        epi, epj = walks.hydro_epi(g, s), walks.hydro_epj(j, s)
        a, b = orc.hydro(epi, epj), orc.hydro(epi, epj, impl="ref")
        for f in ("acch", "accg", "udot", "vsmx", "diffu"):
            assert rel_err(a[f], b[f]).max() < TOL, f
    gi = walks.gravity_epi(groups[0], s)
    gj = walks.gravity_epj(np.arange(n), s)
    a, b = orc.gravity(gi, gj), orc.gravity(gi, gj, impl="ref")
    for f in ("acc", "pot", "eta"):
        assert rel_err(a[f], b[f]).max() < TOL, f


@pytest.mark.skipif(not orc.ref_available(avx2=True), reason="AVX2 reference build absent")
def test_reference_avx2_build_agrees(golden):
    """The reference's AVX2 functors (the timed CPU baseline on x86) agree with
    its scalar FP64 functors to ~1e-12 (4th-order rcp/rsqrt refinement,
    vector_x86.hpp:501-530)."""
    g = golden
    a = slice(0, int(g["dens_i_off"][2]))
    b = slice(0, int(g["dens_j_off"][1]))
    a1 = slice(0, int(g["dens_i_off"][1]))
    out = orc.density(g["dens_epi"][a1], g["dens_epj"][b], impl="ref_avx2")
    ref = g["dens_out"][a1]
    for f in ("dens", "ksr", "grdh"):
        assert rel_err(out[f], ref[f]).max() < 1e-9, f
    del a
