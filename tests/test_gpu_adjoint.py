"""The hand-written derivative of the step (sph_system_adjoint_forces and the
leapfrog reversal in research_codes_gb300.adjoint) against central finite
differences, FP32C against FP64, and through torch.autograd."""
import numpy as np
import pytest

from research_codes_gb300 import abi, adjoint, adjoint_check as chk

pytestmark = pytest.mark.gpu

SCALE = 0.02   # 2 x 1000 particles


@pytest.fixture(scope="module")
def setup():
    """Direct-summation gravity (theta -> 0 opens every node), so that no
    tree opening decision makes the loss jump inside a difference interval."""
    s, eta, R, v_rel = chk.head_on(SCALE, vel_noise=0.02)
    ctx, ps = chk.make_system("fp64", len(s["mass"]), eta, theta=1e-6)
    s0 = chk.converge_h(ps, s)
    yield dict(s=s0, eta=eta, R=R, v_rel=v_rel, ctx=ctx, ps=ps)
    ps.close()
    ctx.close()


def test_force_adjoint_matches_finite_differences(setup):
    """dJ/d(x, v, u, alpha) of J = sum seed . outputs of one force evaluation."""
    ps, s = setup["ps"], setup["s"]
    n = ps.n
    rng = np.random.default_rng(1)
    seed = {"acc": rng.normal(size=(n, 3)), "udot": rng.normal(size=n), "adot": rng.normal(size=n),
            "ksr": 1e-3 * rng.normal(size=n), "pot": rng.normal(size=n), "dens": 1e3 * rng.normal(size=n)}
    base = dict(s)
    base["alph"] = 0.5 + 0.5 * rng.random(n)

    def J(st):
        ps.upload(st)
        ps.compute_forces()
        assert ps.stats()["density_iterations"] == 1
        return sum(float((seed[k] * ps.download(k)).sum()) for k in seed)

    J(base)
    g = ps.adjoint_forces(seed)
    rel_smooth, n_smooth = [], 0
    for i in rng.choice(n, 4, replace=False):
        for key, w, eps in (("pos", 3, 1e-4 * setup["R"]), ("vel", 3, 1e-4 * setup["v_rel"]), ("uene", 1, None),
                            ("alph", 1, None)):
            for c in range(w):
                fds = []
                for sc in (1.0, 0.1):
                    e = (eps if eps else 1e-4 * abs(base[key][i])) * sc
                    st = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in base.items()}
                    idx = (i, c) if w == 3 else i
                    st[key][idx] += e
                    jp = J(st)
                    st[key][idx] -= 2 * e
                    jm = J(st)
                    fds.append((jp - jm) / (2 * e))
                ad = g[key][i, c] if w == 3 else g[key][i]
                den = max(abs(fds[1]), 1e-12)
                if abs(fds[0] - fds[1]) <= 1e-4 * den:
                    n_smooth += 1
                    rel_smooth.append(abs(ad - fds[1]) / den)
    assert n_smooth >= 24, n_smooth
    assert max(rel_smooth) < 1e-4, (max(rel_smooth), np.median(rel_smooth))


def test_bound_mass_gradient_matches_finite_differences(setup):
    """K = 4 steps with a checkpoint every 2; e0 = mean |e| (not saturated)."""
    ps, s = setup["ps"], setup["s"]
    run = adjoint.BoundMassRun(ps, s, steps=4, every=2)
    ps.upload(s)
    ps.compute_forces()
    run.e0 = adjoint.energy_scale(ps, 1.0)
    L = run.forward(s["pos"], s["vel"])
    gx, gv = run.backward()
    assert np.isfinite(L) and np.all(np.isfinite(gx)) and np.all(np.isfinite(gv))
    idx = np.random.default_rng(2).choice(ps.n, 4, replace=False)
    rows = chk.fd_compare(run.forward, s["pos"], s["vel"], gx, gv, idx, 1e-4 * setup["R"], 1e-4 * setup["v_rel"])
    sm = chk.summarise(rows)
    assert sm["smooth"] >= 18, sm
    assert sm["max_rel_smooth"] < 1e-4, (sm, [r for r in rows if r["smooth"] and r["rel"] >= 1e-4])


def test_fp32c_gradient_tracks_fp64(setup):
    s = setup["s"]
    out = {}
    for prec in ("fp64", "fp32c"):
        ctx, ps = chk.make_system(prec, len(s["mass"]), setup["eta"])
        run = adjoint.BoundMassRun(ps, s, steps=3, every=2, dt=2.0, e0=2.0)
        L = run.forward(s["pos"], s["vel"])
        out[prec] = (L,) + run.backward()
        ps.close()
        ctx.close()
    (L64, x64, v64), (L32, x32, v32) = out["fp64"], out["fp32c"]
    assert abs(L32 - L64) <= 1e-6 * abs(L64)
    assert np.linalg.norm(x32 - x64) <= 1e-4 * np.linalg.norm(x64)
    assert np.linalg.norm(v32 - v64) <= 1e-4 * np.linalg.norm(v64)


def test_torch_autograd_function(setup):
    torch = pytest.importorskip("torch")
    ps, s = setup["ps"], setup["s"]
    run = adjoint.BoundMassRun(ps, s, steps=2, every=1, dt=2.0, e0=2.0)
    BoundMass = adjoint.autograd_function()
    x0 = torch.tensor(s["pos"], requires_grad=True)
    v0 = torch.tensor(s["vel"], requires_grad=True)
    L = BoundMass.apply(x0, v0, run)
    (3.0 * L).backward()
    L2 = run.forward(s["pos"], s["vel"])
    gx, gv = run.backward()
    assert abs(L.item() - L2) <= 1e-12 * abs(L2)
    assert np.allclose(x0.grad.numpy(), 3.0 * gx, rtol=1e-12, atol=0)
    assert np.allclose(v0.grad.numpy(), 3.0 * gv, rtol=1e-12, atol=0)


def test_adjoint_refuses_what_it_does_not_cover(setup):
    s = setup["s"]
    ctx, ps = chk.make_system("fp64", len(s["mass"]), setup["eta"])
    ps.set_params(alphu_max=1.0)
    ps.upload(s)
    ps.compute_forces()
    with pytest.raises(abi.SPHError):
        ps.adjoint_forces({"acc": np.zeros((ps.n, 3))})
    ps.close()
    ctx.close()


def test_config3_tree_gravity_gradient_matches_finite_differences():
    """The differentiable-step configuration scaled to 2 x 5k particles:
    theta = 0.5 tree gravity (not direct summation), K = 20 leapfrog steps
    with a checkpoint every 5, loss sum m sigmoid(-e/e0) with e0 the mean
    |e| (1% of it saturates the sigmoid: the gradient is exactly 0).  Central
    differences at eps = 1e-4 R (positions) and 1e-4 v_rel (velocities) and
    at eps/10 on 8 random particles; where the two agree to 1e-4 no opening
    decision or switch changes inside the interval and the adjoint must match
    to 1e-4."""
    s, eta, R, v_rel = chk.head_on(0.1)
    ctx, ps = chk.make_system("fp64", len(s["mass"]), eta, theta=0.5)
    try:
        s0 = chk.converge_h(ps, s)
        run = adjoint.BoundMassRun(ps, s0, steps=20, every=5)
        ps.upload(s0)
        ps.compute_forces()
        run.e0 = adjoint.energy_scale(ps, 1.0)
        L = run.forward(s0["pos"], s0["vel"])
        gx, gv = run.backward()
        assert np.isfinite(L) and np.all(np.isfinite(gx)) and np.all(np.isfinite(gv))
        idx = np.random.default_rng(5).choice(ps.n, 8, replace=False)
        rows = chk.fd_compare(run.forward, s0["pos"], s0["vel"], gx, gv, idx, 1e-4 * R, 1e-4 * v_rel)
        sm = chk.summarise(rows)
        assert sm["smooth"] >= 24, sm
        assert sm["max_rel_smooth"] < 1e-4, (sm, [r for r in rows if r["smooth"] and r["rel"] >= 1e-4])
    finally:
        ps.close()
        ctx.close()
