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


# ---- per-particle step glue ------------------------------------------------------
GLUE = "glue_n256.npz"


@pytest.fixture(scope="module")
def glue():
    import os
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", GLUE)))


def _glue_oracle(g):
    """The C restatement on the golden inputs, named like the golden outputs."""
    i = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    o = {}
    o["pres"], o["vsnd"] = orc.eos(i["dens"], i["uene"])
    o["bswt"] = orc.balsara(i["divv"], i["rotv"], o["vsnd"], i["ksr"])
    o["adot"], _ = orc.alpha_dot(i["divv"], i["alph"], i["alphu"], o["vsnd"], i["ksr"], i["uene"],
                                 np.zeros_like(i["uene"]), float(g["alpha_max"]), float(g["alpha_min"]), 0.0, 0.0,
                                 1.0)
    vsmx = g["ref_vsmx_in"]
    c_dt, dt_max = float(g["c_dt"]), float(g["dt_max"])
    o["dt_min"] = orc.timestep_min(i["ksr"], vsmx, i["divv"], i["accg1"] + i["accg2"], c_dt, dt_max)
    o["energy"] = orc.energy(i["mass"], i["vel"], i["uene"], i["pot"])[0]
    dt = float(i["dt"])
    p = orc.predict(dt, i)
    for k, v in p.items():
        o["pred_" + k] = v
    new = dict(p, acc=i["acc"][::-1], udot=i["udot"][::-1], adot=i["adot"][::-1], adotu=i["adotu"])
    for k, v in orc.correct(dt, new).items():
        o["corr_" + k] = v
    o["acc_sum"] = orc.sum_acceleration(i["acch"], i["accg1"], i["accg2"])
    o["ksrmax"] = orc.ksrmax(i["mass"], i["pos"], i["vel"], i["istar"], i["dens"])
    return o


def test_glue_matches_reference_golden(glue):
    """EOS, Balsara switch, alpha derivative, time step, energy, predictor,
    corrector, sumAcceleration and ksrmax of the restatement against the
    reference's own glue (hdr_hgas.hpp, hdr_sph.hpp, hdr_util.hpp) on the
    same inputs: identical formulas in FP64, so identical to rounding."""
    g = glue
    o = _glue_oracle(g)
    for k in ("pres", "vsnd", "bswt", "adot", "pred_pos", "pred_vel", "pred_vel2", "pred_uene", "pred_uene2",
              "pred_alph", "pred_alph2", "pred_alphu", "pred_alphu2", "corr_vel", "corr_uene", "corr_alph",
              "corr_alphu", "acc_sum"):
        assert rel_err(o[k], g["ref_" + k], 1e-12).max() <= 1e-14, k
    # the particles' minimum step and the energy sum in index order
    assert o["dt_min"] == pytest.approx(min(float(g["dt_max"]), g["ref_dt_particle"].min()), rel=1e-15)
    e_ref = 0.0
    for e in g["ref_energy_particle"]:
        e_ref += e
    assert o["energy"] == pytest.approx(e_ref, rel=1e-14)
    assert float(o["ksrmax"]) == pytest.approx(float(g["ref_ksrmax"]), rel=1e-14)
    # the inputs reach every branch: compression and none, both stars
    assert (g["in_divv"] == 0).any() and (g["in_divv"] < 0).any() and (g["in_istar"] == 0).any()


@pytest.mark.skipif(not orc.ref_glue_available(), reason="oracle/_ref/libsph_ref_glue.so not built here")
def test_glue_golden_is_the_live_reference(glue):
    """The stored outputs are what the reference's glue computes now."""
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "make_glue_golden", os.path.join(os.path.dirname(__file__), "golden", "make_glue_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    live = mk.reference_outputs(mk.inputs())
    for k, v in live.items():
        assert np.array_equal(v, glue["ref_" + k]), k


def test_timestep_pow2_known_answers():
    """main.cpp:242-273: halve while dt > dtc, abort at dt_min; double only
    when 2 dt fits under dtc and dt_max and the time is a multiple of 2 dt."""
    f = orc.timestep_pow2
    assert f(10.0, 3.0, 0.0, 10.0, 1e-6) == 2.5          # 10 -> 5 -> 2.5
    assert f(2.5, 7.0, 5.0, 10.0, 1e-6) == 5.0           # 5 is a multiple of 5
    assert f(2.5, 7.0, 7.5, 10.0, 1e-6) == 2.5           # 7.5 is not
    assert f(5.0, 12.0, 10.0, 10.0, 1e-6) == 10.0        # 2 dt == dt_max is allowed
    assert f(5.0, 12.0, 10.0, 9.0, 1e-6) == 5.0          # 2 dt above dt_max
    assert f(2.5, 2.5, 0.0, 10.0, 1e-6) == 2.5           # dt == dtc: kept
    assert f(1.0, 1e-9, 0.0, 10.0, 1e-6) < 0             # would fall to dt_min: the reference aborts
