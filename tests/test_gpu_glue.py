"""The per-particle step glue of the device engine against the oracle's FP64
restatement (oracle/sph_oracle.c, itself pinned to the reference's own glue
by tests/test_oracle.py): EOS and Balsara switch (hdr_hgas.hpp:339-342,
hdr_sph.hpp:79-89), sumAcceleration (hdr_sph.hpp:95-97), the alpha
derivatives (hdr_hgas.hpp:750-762), ksrmax (hdr_util.hpp:489-527), the total
energy (main.cpp:199-219), the power-of-two time step (hdr_hgas.hpp:477-488,
main.cpp:242-273) and one predictor + corrector (hdr_hgas.hpp:646-665).

Inputs of each oracle call are the device's own fields of the same
evaluation, so every comparison isolates one piece of glue.  FP64 runs match
to 1e-12; FP32C runs compute the sound speed, Balsara switch, alpha damping
and the time-step candidates in FP32 arithmetic (they feed FP32 records) and
match to 1e-5; the integration itself is FP64 in both."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as orc
from research_codes_gb300 import functors, ic
from research_codes_gb300.system import ParticleSystem, state_from_ic

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "mass", "uene", "dens", "pres", "vsnd", "bswt", "divv", "rotv", "ksr", "alph", "alphu",
          "adot", "adotu", "diffu", "acc", "acch", "accg1", "accg2", "vsmx", "udot", "pot", "istar")


def _states():
    c0, eta0 = ic.config_system("c0")
    c0 = state_from_ic(c0)
    rng = np.random.default_rng(11)
    c0["vel"] = np.cross([0.0, 0.0, 2e-3], c0["pos"]) + rng.normal(scale=2.0, size=c0["pos"].shape)
    a = ic.polytrope(7200, 10.0, 4.0, 3.0, seed=21, eta=1.18)
    b = ic.polytrope(4800, 3.0, 1.5, 1.5, seed=22, eta=1.18)
    sep = 1.5 * (a["R"] + b["R"])
    two = state_from_ic(ic.two_stars(a, b, sep, 0.5 * (a["R"] + b["R"]), 1.2 * ic.escape_speed(a["M"] + b["M"], sep)))
    return {"c0-10k": (c0, eta0), "two-stars-12k": (two, 1.18)}


STATES = _states()


@pytest.fixture(scope="module", params=[(p, k) for k in STATES for p in ("fp64", "fp32c")],
                ids=lambda t: f"{t[0]}-{t[1]}")
def stepped(request):
    """A state evaluated once (eager), then advanced by one eager step; the
    fields and clock before and after."""
    prec, key = request.param
    s, eta = STATES[key]
    ctx = functors.Context(precision=prec, eta=eta, ksr_max=0.0)
    sys = ParticleSystem(ctx, len(s["mass"]), n_group=64, use_graph=0, ksr_max_mode=1)
    sys.upload(s)
    sys.compute_forces()
    before = {k: sys.download(k) for k in FIELDS}
    clk0, st0 = sys.clock(), sys.stats()
    sys.step(1)
    after = {k: sys.download(k) for k in FIELDS}
    clk1, st1 = sys.clock(), sys.stats()
    yield dict(prec=prec, b=before, a=after, clk0=clk0, clk1=clk1, st0=st0, st1=st1, prm=sys.params)
    sys.close()
    ctx.close()


def _tol(d, fp32_glue=False):
    return 1e-5 if (fp32_glue and d["prec"] == "fp32c") else 1e-12


def test_eos_and_balsara(stepped):
    """On the evaluated state before the step (after it, u and alpha hold the
    corrector's values, not those the evaluation used)."""
    d = stepped
    f = d["b"]
    pres, vsnd = orc.eos(f["dens"], f["uene"])
    assert rel_err(f["pres"], pres).max() < 1e-14
    assert rel_err(f["vsnd"], vsnd).max() < _tol(d, True)
    bswt = orc.balsara(f["divv"], f["rotv"], vsnd, f["ksr"])
    assert rel_err(f["bswt"], bswt).max() < _tol(d, True)


def test_sum_acceleration(stepped):
    for f in (stepped["b"], stepped["a"]):
        assert np.array_equal(f["acc"], orc.sum_acceleration(f["acch"], f["accg1"], f["accg2"]))


def test_alpha_derivatives(stepped):
    d = stepped
    f, p = d["b"], d["prm"]
    eps_u = d["clk0"][3]
    adot, adotu = orc.alpha_dot(f["divv"], f["alph"], f["alphu"], f["vsnd"], f["ksr"], f["uene"], f["diffu"],
                                p.alpha_max, p.alpha_min, p.alphu_max, p.alphu_min, eps_u)
    # alpha' = -(alpha - alpha_min) / tau + source is a difference of two
    # terms: FP32C's FP32 damping rate is judged against 1e-3 of the field's
    # largest value, as the other derived fields
    floor = 1e-6 if d["prec"] == "fp64" else 1e-3
    assert rel_err(f["adot"], adot, floor).max() < _tol(d, True)
    assert rel_err(f["adotu"], adotu, floor).max() < _tol(d, True)


def test_ksrmax_and_energy(stepped):
    d = stepped
    for f, clk, st in ((d["b"], d["clk0"], d["st0"]), (d["a"], d["clk1"], d["st1"])):
        km = orc.ksrmax(f["mass"], f["pos"], f["vel"], f["istar"], f["dens"])
        assert clk[2] == pytest.approx(km, rel=1e-12)
    # the energy of the stepped state (reduced after its corrector)
    f = d["a"]
    e, ek, eu, ep = orc.energy(f["mass"], f["vel"], f["uene"], f["pot"])
    st = d["st1"]
    assert st["e_tot"] == pytest.approx(e, rel=1e-12)
    assert (st["e_kin"], st["e_thm"], st["e_pot"]) == pytest.approx((ek, eu, ep), rel=1e-12)


def test_power_of_two_time_step(stepped):
    d = stepped
    f, p = d["b"], d["prm"]
    t0, dt0 = d["clk0"][0], d["clk0"][1]
    dtc = orc.timestep_min(f["ksr"], f["vsmx"], f["divv"], f["accg1"] + f["accg2"], p.c_dt, p.dt_max)
    dt = orc.timestep_pow2(dt0, dtc, t0, p.dt_max, p.dt_min)
    assert dt > 0
    # the step's dt is a power-of-two fraction: identical unless FP32 time-step
    # candidates put dtc within their rounding of a halving threshold
    if d["prec"] == "fp64":
        assert d["clk1"][1] == dt
    else:
        assert d["clk1"][1] in (dt, 0.5 * dt, 2.0 * dt)
    assert d["clk1"][0] == t0 + d["clk1"][1]


def test_predict_and_correct(stepped):
    """Positions after the step are the predictor's (the corrector leaves
    them); velocity, u and alpha are the corrector's, from the predictor's
    half-step values and the derivatives of the step's force evaluation."""
    d = stepped
    b, a = d["b"], d["a"]
    dt = d["clk1"][1]
    pred = orc.predict(dt, b)
    disp, disp_ref = a["pos"] - b["pos"], pred["pos"] - b["pos"]
    assert rel_err(disp, disp_ref, 1e-6).max() < 1e-12
    corr = orc.correct(dt, dict(pred, acc=a["acc"], udot=a["udot"], adot=a["adot"], adotu=a["adotu"]))
    assert rel_err(a["vel"] - b["vel"], corr["vel"] - b["vel"], 1e-6).max() < 1e-12
    assert rel_err(a["uene"], corr["uene"]).max() < 1e-14
    assert rel_err(a["alph"], corr["alph"]).max() < 1e-14
    assert rel_err(a["alphu"], corr["alphu"], 1e-6).max() < 1e-12
