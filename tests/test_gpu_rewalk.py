"""The search-radius re-walk loop of the density (calcDensityKernel,
hdr_density.hpp:372-415) against the oracle, walk by walk.

The state starts from 0.9 x its converged smoothing lengths h, so the first
walk (rs = 1.1 h0 = 0.99 h) leaves the particles whose new h grew beyond their
search radius iterating, and a second walk (rs = 1.21 h0 = 1.089 h, the same
first guess h0) finishes them.  The oracle replays both walks on the engine's own exported
lists (kind 0: the first walk; kind 3: the last re-walk) with the same first
guess and search radii: every particle's final density, h, grad-h term,
div v, |rot v| and neighbour count come from the walk in which it stopped
iterating, and the set of particles re-walked is the oracle's.

A second case starts only 24 particles from 0.85 x their converged h, so
the re-walk has at most 1024 iterating particles and runs on the
block-per-walk kernel (density_rewalk_blocks) instead of density_kernel."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as orc
from research_codes_gb300 import abi, functors, ic, walks
from research_codes_gb300.system import ParticleSystem, state_from_ic

pytestmark = pytest.mark.gpu

FIELDS = ("dens", "ksr", "grdh", "divv", "rotv")
DERIV = ("divv", "rotv")


def _state():
    a = ic.polytrope(3600, 10.0, 4.0, 3.0, seed=31, eta=1.18)
    b = ic.polytrope(2400, 3.0, 1.5, 1.5, seed=32, eta=1.18)
    sep = 1.3 * (a["R"] + b["R"])
    s = state_from_ic(ic.two_stars(a, b, sep, 0.4 * (a["R"] + b["R"]), 1.2 * ic.escape_speed(a["M"] + b["M"], sep)))
    rng = np.random.default_rng(5)
    s["vel"] = s["vel"] + rng.normal(scale=3.0, size=s["vel"].shape)
    return s


@pytest.mark.parametrize("few", [False, True])
@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_density_rewalk_matches_oracle_walk_by_walk(prec, few):
    s = _state()
    n = len(s["mass"])
    ctx = functors.Context(precision=prec, eta=1.18, ksr_max=0.0)
    sys = ParticleSystem(ctx, n, n_group=64, use_graph=0, ksr_max_mode=0)
    try:
        sys.upload(s)
        sys.compute_forces()
        sys.compute_forces()
        if few:
            s["ksr"] = sys.download("ksr")
            pick = np.random.default_rng(7).choice(n, 24, replace=False)
            s["ksr"][pick] *= 0.85
        else:
            s["ksr"] = 0.9 * sys.download("ksr")
        sys.upload(s)
        sys.compute_forces()
        st = sys.stats()
        assert st["density_iterations"] == 2, st["density_iterations"]
        f = {k: sys.download(k, sorted_order=True) for k in ("pos", "vel", "mass", "id", "np") + FIELDS}
        order = sys.download("id", sorted_order=True).astype(np.int64)
        h0 = np.empty(n)
        h0[:] = s["ksr"][order]                     # ids are upload indices here
        state = dict(pos=f["pos"], vel=f["vel"], mass=f["mass"], id=f["id"].astype(np.int64), ksr=h0)

        # walk 0: every group, rs = 1.1 h0
        out = np.zeros(n, abi.Density)
        state["rs"] = 1.1 * h0
        i_first, i_count, j_off, j_idx = sys.lists(0)
        for w in range(len(i_first)):
            gi = np.arange(i_first[w], i_first[w] + i_count[w])
            out[gi] = orc.density(walks.density_epi(gi, state), walks.density_epj(j_idx[j_off[w]:j_off[w + 1]], state),
                                  eta=1.18, ksr_max=0.0)
        again = out["itr"].astype(bool)
        assert 0 < again.sum() < n
        if few:
            assert again.sum() <= 1024     # the block-per-walk re-walk

        # walk 1: the groups holding iterating particles, rs = 1.21 h0, those particles only
        state["rs"] = 1.1 * 1.1 * h0
        i_first, i_count, j_off, j_idx = sys.lists(3)
        seen = np.zeros(n, bool)
        for w in range(len(i_first)):
            grp = np.arange(i_first[w], i_first[w] + i_count[w])
            gi = grp[again[grp]]
            assert len(gi) > 0
            seen[gi] = True
            o1 = orc.density(walks.density_epi(gi, state), walks.density_epj(j_idx[j_off[w]:j_off[w + 1]], state),
                             eta=1.18, ksr_max=0.0)
            assert not o1["itr"].any()            # the second walk finishes them
            out[gi] = o1
        assert np.array_equal(seen, again)

        tol = 1e-11 if prec == "fp64" else 1e-5
        for k in FIELDS:
            e = rel_err(f[k], out[k], 1e-2 if k in DERIV else 1e-3).max()
            assert e < (tol if k not in DERIV or prec == "fp64" else 1e-4), (k, e)
        dnp = np.abs(f["np"].astype(np.int64) - out["np"]).max()
        assert dnp <= (0 if prec == "fp64" else 1), dnp
    finally:
        sys.close()
        ctx.close()
