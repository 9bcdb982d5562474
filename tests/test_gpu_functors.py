"""GPU parity of the three functors and the multiwalk Dispatch/Retrieve pairs
against the reference's outputs (golden vectors) and the oracle (fresh seeded
inputs), in both precisions.

Tolerances (relative, per particle; vector fields by norm):
  FP64 mode   : 1e-11 on every real field (same arithmetic, different order).
  FP32C mode  : 1e-5 on rho, h, Omega (grdh), a (hydro, softening correction
                accg, gravity), du/dt, pot, eta, v_sig (the hydro sums that
                cancel are formed in double-float); 1e-4 on div v, |rot v| and
                the conduction signal diffu, FP32 sums of strongly cancelling
                neighbour terms.  Per-particle errors are floored at 1e-3 of
                the field's largest magnitude (1e-2 for div v, |rot v|,
                diffu), so a particle whose vector nearly cancels (symmetric
                neighbourhood) is measured against the field's scale.  np and
                itr must match except where a neighbour sits at q = 1 within
                FP32 rounding (at most 1% of particles).
"""
import numpy as np
import pytest

from conftest import rel_err, walk_slices
from oracle import oracle as orc
from research_codes_gb300 import abi, functors, walks

pytestmark = pytest.mark.gpu

TOL64 = 1e-11
TOL32 = 1e-5
TOL32_DERIV = 1e-4
FLOOR = 1e-3
FLOOR_DERIV = 1e-2


def err(a, b, floor=FLOOR):
    return rel_err(a, b, floor_frac=floor).max()


@pytest.fixture(scope="module", params=["fp32c", "fp64"])
def ctx(request):
    c = functors.Context(precision=request.param)
    c.mode = request.param
    yield c
    c.close()


def _tol(ctx, deriv=False):
    if ctx.mode == "fp64":
        return TOL64
    return TOL32_DERIV if deriv else TOL32


def check_density(ctx, out, ref):
    for f in ("dens", "ksr", "grdh"):
        assert err(out[f], ref[f]) < _tol(ctx), (f, err(out[f], ref[f]))
    for f in ("divv", "rotv"):
        assert err(out[f], ref[f], FLOOR_DERIV) < _tol(ctx, True), (f, err(out[f], ref[f], FLOOR_DERIV))
    if ctx.mode == "fp64":
        assert np.array_equal(out["np"], ref["np"])
        assert np.array_equal(out["itr"], ref["itr"])
    else:
        assert np.mean(out["np"] != ref["np"]) <= 0.01
        assert np.abs(out["np"] - ref["np"]).max() <= 1
        assert np.mean(out["itr"] != ref["itr"]) <= 0.01


def check_hydro(ctx, out, ref):
    for f in ("acch", "accg", "udot", "vsmx"):
        assert err(out[f], ref[f]) < _tol(ctx), (f, err(out[f], ref[f]))
    assert err(out["diffu"], ref["diffu"], FLOOR_DERIV) < _tol(ctx, True), err(out["diffu"], ref["diffu"], FLOOR_DERIV)


def check_gravity(ctx, out, ref):
    for f in ("acc", "pot", "eta"):
        assert err(out[f], ref[f]) < _tol(ctx), (f, err(out[f], ref[f]))


# ---- golden vectors (reference outputs) ---------------------------------------

def test_density_golden(ctx, golden):
    g = golden
    f = functors.calcDensity(ctx)
    ctx.set_ksr_max(0.0)
    for _, a, b in walk_slices(g["dens_i_off"], g["dens_j_off"]):
        epi, epj = g["dens_epi"][a].copy(), g["dens_epj"][b].copy()
        out = np.zeros(len(epi), abi.Density)
        f(epi, len(epi), epj, len(epj), out)
        check_density(ctx, out, g["dens_out"][a])


def test_density_clamp_golden(ctx, golden):
    g = golden
    ctx.set_ksr_max(float(g["densc_ksr_max"]))
    try:
        f = functors.calcDensity(ctx)
        for _, a, b in walk_slices(g["densc_i_off"], g["densc_j_off"]):
            epi, epj = g["densc_epi"][a].copy(), g["densc_epj"][b].copy()
            out = np.zeros(len(epi), abi.Density)
            f(epi, len(epi), epj, len(epj), out)
            check_density(ctx, out, g["densc_out"][a])
    finally:
        ctx.set_ksr_max(0.0)


def test_hydro_golden(ctx, golden):
    g = golden
    f = functors.calcHydro(ctx)
    for _, a, b in walk_slices(g["hydro_i_off"], g["hydro_j_off"]):
        epi, epj = g["hydro_epi"][a].copy(), g["hydro_epj"][b].copy()
        out = np.zeros(len(epi), abi.Hydro)
        f(epi, len(epi), epj, len(epj), out)
        check_hydro(ctx, out, g["hydro_out"][a])


def test_gravity_golden_two_calls_accumulate(ctx, golden):
    """EPJ call then SPJ call into one cleared force, as FDPS does."""
    g = golden
    f = functors.calcGravity(ctx)
    io, jo, so = g["grav_i_off"], g["grav_j_off"], g["grav_s_off"]
    for w in range(len(io) - 1):
        epi = g["grav_epi"][io[w]:io[w + 1]].copy()
        epj = g["grav_epj"][jo[w]:jo[w + 1]].copy()
        spj = g["grav_spj"][so[w]:so[w + 1]].copy()
        out = np.zeros(len(epi), abi.Gravity)
        f(epi, len(epi), epj, len(epj), out)
        f(epi, len(epi), spj, len(spj), out)
        check_gravity(ctx, out, g["grav_out"][io[w]:io[w + 1]])


def test_multiwalk_dispatch_retrieve_golden(ctx, golden):
    g = golden
    io, jo = g["dens_i_off"], g["dens_j_off"]
    nw = len(io) - 1
    epi = [g["dens_epi"][io[w]:io[w + 1]].copy() for w in range(nw)]
    epj = [g["dens_epj"][jo[w]:jo[w + 1]].copy() for w in range(nw)]
    outs = [np.zeros(len(a), abi.Density) for a in epi]
    functors.DispatchKernel_Dens(ctx, 0, nw, epi, [len(a) for a in epi], epj, [len(b) for b in epj])
    functors.RetrieveKernel_Dens(ctx, 0, nw, [len(a) for a in epi], outs)
    check_density(ctx, np.concatenate(outs), g["dens_out"])

    io, jo, so = g["grav_i_off"], g["grav_j_off"], g["grav_s_off"]
    nw = len(io) - 1
    gi = [g["grav_epi"][io[w]:io[w + 1]].copy() for w in range(nw)]
    gj = [g["grav_epj"][jo[w]:jo[w + 1]].copy() for w in range(nw)]
    gs = [g["grav_spj"][so[w]:so[w + 1]].copy() for w in range(nw)]
    gout = [np.full(len(a), 7, abi.Gravity) for a in gi]      # retrieve assigns
    functors.DispatchKernel_Gravity(ctx, 0, nw, gi, [len(a) for a in gi], gj, [len(b) for b in gj],
                                    gs, [len(c) for c in gs])
    functors.RetrieveKernel_Gravity(ctx, 0, nw, [len(a) for a in gi], gout)
    check_gravity(ctx, np.concatenate(gout), g["grav_out"])

    io, jo = g["hydro_i_off"], g["hydro_j_off"]
    nw = len(io) - 1
    hi = [g["hydro_epi"][io[w]:io[w + 1]].copy() for w in range(nw)]
    hj = [g["hydro_epj"][jo[w]:jo[w + 1]].copy() for w in range(nw)]
    hout = [np.zeros(len(a), abi.Hydro) for a in hi]
    functors.DispatchKernel_HydroForce(ctx, 0, nw, hi, [len(a) for a in hi], hj, [len(b) for b in hj])
    functors.RetrieveKernel_HydroForce(ctx, 0, nw, [len(a) for a in hi], hout)
    check_hydro(ctx, np.concatenate(hout), g["hydro_out"])


# ---- fresh seeded inputs against the oracle -----------------------------------

def _collision_system(seed, n=3000):
    """Two offset blobs moving towards each other at high bulk speed: FP32
    coordinates far from the origin and large common velocities test the
    group-centred arithmetic."""
    rng = np.random.default_rng(seed)
    a = rng.normal(size=(n // 2, 3))
    b = rng.normal(size=(n - n // 2, 3)) * 0.7 + np.array([2.5, 0.4, 0.0])
    pos = np.concatenate([a, b]) + 3.0e4                         # far from the origin
    vel = np.concatenate([np.tile([400.0, 0, 0], (n // 2, 1)), np.tile([-400.0, 0, 0], (n - n // 2, 1))])
    vel += rng.normal(scale=1.0, size=vel.shape)
    mass = rng.uniform(0.8, 1.2, n) / n
    rho_est = np.exp(-0.5 * (np.linalg.norm(pos - pos.mean(0), axis=1) ** 2)) + 0.05
    h = 1.2 * 1.936492 * (mass / (rho_est / n * n)) ** (1 / 3) * 0.25
    s = dict(pos=pos, vel=vel, mass=mass, ksr=h, rs=1.1 * h, id=rng.permutation(n).astype(np.int64))
    return s, rng


@pytest.mark.parametrize("seed", [11, 12])
def test_density_vs_oracle_collision(ctx, seed):
    """Errors measured over all walks together (the field's own scale)."""
    s, _ = _collision_system(seed)
    groups = walks.make_groups(s["pos"], 100)
    jl = walks.gather_lists(s["pos"], s["rs"], groups)
    ctx.set_eta(1.2)
    outs, refs = [], []
    try:
        f = functors.calcDensity(ctx)
        for g, j in list(zip(groups, jl))[::2]:
            epi, epj = walks.density_epi(g, s), walks.density_epj(j, s)
            out = np.zeros(len(epi), abi.Density)
            f(epi, len(epi), epj, len(epj), out)
            outs.append(out)
            refs.append(orc.density(epi, epj, eta=1.2))
    finally:
        ctx.set_eta(1.6)
    check_density(ctx, np.concatenate(outs), np.concatenate(refs))


def test_hydro_gravity_vs_oracle_collision(ctx):
    s, rng = _collision_system(13)
    n = len(s["mass"])
    s.update(pres=rng.uniform(1, 2, n) * 1e-3, grdh=rng.uniform(0.8, 1.2, n),
             dens=rng.uniform(1, 3, n), bswt=rng.uniform(0, 1, n), vsnd=rng.uniform(1, 2, n) * 50,
             alph=rng.uniform(0.1, 2, n), alphu=rng.uniform(0, 1, n),
             uene=rng.uniform(1, 2, n) * 1e3, eta=rng.uniform(0, 0.3, n))
    groups = walks.make_groups(s["pos"], 64)
    hl = walks.symmetric_lists(s["pos"], s["ksr"], groups)
    fh = functors.calcHydro(ctx)
    outs, refs = [], []
    for g, j in list(zip(groups, hl))[::5]:
        epi, epj = walks.hydro_epi(g, s), walks.hydro_epj(j, s)
        out = np.zeros(len(epi), abi.Hydro)
        fh(epi, len(epi), epj, len(epj), out)
        outs.append(out)
        refs.append(orc.hydro(epi, epj))
    check_hydro(ctx, np.concatenate(outs), np.concatenate(refs))
    fg = functors.calcGravity(ctx)
    eps2 = (s["ksr"] / 1.936492) ** 2
    el, sl = walks.gravity_lists(s["pos"], s["mass"], eps2, groups, near_factor=1.0, cell_frac=0.1)
    outs, refs = [], []
    for g, e, sp in list(zip(groups, el, sl))[::7]:
        epi, epj = walks.gravity_epi(g, s), walks.gravity_epj(e, s)
        out = np.zeros(len(epi), abi.Gravity)
        fg(epi, len(epi), epj, len(epj), out)
        fg(epi, len(epi), sp, len(sp), out)
        outs.append(out)
        refs.append(orc.gravity(epi, epj, sp))
    check_gravity(ctx, np.concatenate(outs), np.concatenate(refs))


# ---- edge cases ---------------------------------------------------------------

def test_ragged_and_empty_walks(ctx, golden):
    """Walks with 0 i-particles, 1 i-particle, and 33 (two work items)."""
    g = golden
    epj = g["dens_epj"][: int(g["dens_j_off"][1])].copy()
    base = g["dens_epi"][: int(g["dens_i_off"][1])].copy()
    sizes = [0, 1, 33, min(len(base), 64)]
    epi = [base[:k].copy() for k in sizes]
    outs = [np.zeros(k, abi.Density) for k in sizes]
    functors.DispatchKernel_Dens(ctx, 0, len(sizes), epi, sizes, [epj] * len(sizes), [len(epj)] * len(sizes))
    functors.RetrieveKernel_Dens(ctx, 0, len(sizes), sizes, outs)
    for k, o in zip(sizes, outs):
        if k:
            check_density(ctx, o, orc.density(base[:k], epj))


def test_zero_walks_is_a_no_op(ctx):
    functors.DispatchKernel_Dens(ctx, 0, 0, [], [], [], [])
    functors.RetrieveKernel_Dens(ctx, 0, 0, [], [])


def test_gravity_functor_accumulates(ctx, golden):
    g = golden
    epi = g["grav_epi"][: int(g["grav_i_off"][1])].copy()
    epj = g["grav_epj"][: int(g["grav_j_off"][1])].copy()
    f = functors.calcGravity(ctx)
    once = np.zeros(len(epi), abi.Gravity)
    f(epi, len(epi), epj, len(epj), once)
    twice = once.copy()
    f(epi, len(epi), epj, len(epj), twice)
    assert rel_err(twice["pot"], 2 * once["pot"]).max() < 1e-12


def test_capacity_and_state_errors(golden):
    g = golden
    # the truncated j-lists below give rho = 0 (NaN outputs) by design
    with functors.Context(max_walks=2, max_j=100, check_finite=False) as c:
        epi = g["dens_epi"][:4].copy()
        epj = g["dens_epj"][:200].copy()
        with pytest.raises(abi.SPHError) as e:
            functors.DispatchKernel_Dens(c, 0, 3, [epi] * 3, [4] * 3, [epj[:10]] * 3, [10] * 3)
        assert e.value.status == abi.SPH_ERR_CAPACITY
        with pytest.raises(abi.SPHError) as e:
            functors.DispatchKernel_Dens(c, 0, 1, [epi], [4], [epj], [200])
        assert e.value.status == abi.SPH_ERR_CAPACITY
        with pytest.raises(abi.SPHError) as e:
            functors.RetrieveKernel_Dens(c, 0, 1, [4], [np.zeros(4, abi.Density)])
        assert e.value.status == abi.SPH_ERR_STATE
        # a second dispatch before the retrieve is out of sequence
        functors.DispatchKernel_Dens(c, 0, 1, [epi], [4], [epj[:50]], [50])
        with pytest.raises(abi.SPHError) as e:
            functors.DispatchKernel_Dens(c, 0, 1, [epi], [4], [epj[:50]], [50])
        assert e.value.status == abi.SPH_ERR_STATE
        out = np.zeros(4, abi.Density)
        functors.RetrieveKernel_Dens(c, 0, 1, [4], [out])


def test_nonfinite_input_is_reported(golden):
    """A NaN position propagates to the outputs and is reported, not hidden."""
    g = golden
    epi = g["dens_epi"][:8].copy()
    epj = g["dens_epj"][: int(g["dens_j_off"][1])].copy()
    epj["pos"][3] = np.nan
    with functors.Context() as c:
        out = np.zeros(len(epi), abi.Density)
        with pytest.raises(abi.SPHError) as e:
            functors.calcDensity(c)(epi, len(epi), epj, len(epj), out)
        assert e.value.status == abi.SPH_ERR_NONFINITE
