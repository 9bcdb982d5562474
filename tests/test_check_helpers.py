"""CPU tests of the helpers behind the derivative checks and the
configuration runs: central differences and their smoothness test, and the
floored per-particle error statistics."""
import numpy as np

from research_codes_gb300 import adjoint_check, run_configs


def _quadratic(a, b):
    def f(x, v):
        return float((a * x * x).sum() + (b * v * v).sum())
    return f


def test_fd_compare_matches_an_exact_gradient():
    rng = np.random.default_rng(1)
    x0, v0 = rng.normal(size=(5, 3)), rng.normal(size=(5, 3))
    a, b = rng.uniform(0.5, 2.0, size=(5, 3)), rng.uniform(0.5, 2.0, size=(5, 3))
    f = _quadratic(a, b)
    gx, gv = 2 * a * x0, 2 * b * v0
    rows = adjoint_check.fd_compare(f, x0, v0, gx, gv, [0, 3], 1e-3, 1e-3)
    assert len(rows) == 12
    assert all(r["smooth"] for r in rows)
    s = adjoint_check.summarise(rows)
    assert s["smooth"] == 12 and s["max_rel_smooth"] < 1e-7


def test_fd_compare_flags_a_kink_as_not_smooth():
    # |x| at x = 0: the two step sizes agree (both 0), but a kink between the
    # steps (x just off 0) makes the coarse and fine differences disagree
    def f(x, v):
        return float(np.abs(x[0, 0] - 2e-4) + (v * v).sum())
    x0, v0 = np.zeros((1, 3)), np.ones((1, 3))
    gx, gv = np.zeros((1, 3)), 2 * v0
    rows = adjoint_check.fd_compare(f, x0, v0, gx, gv, [0], 1e-3, 1e-3)
    row = [r for r in rows if r["c"] == "x"][0]
    assert not row["smooth"]
    assert all(r["smooth"] for r in rows if r["c"].startswith("v"))
    s = adjoint_check.summarise(rows)
    assert s["smooth"] == len(rows) - 1


def test_rel_stats_floor_and_vectors():
    ref = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 2.0, 0.0]])
    got = ref + np.array([[1e-6, 0.0, 0.0], [1e-9, 0.0, 0.0], [0.0, 0.0, 0.0]])
    s = run_configs.rel_stats(got, ref, floor=1e-3)
    # the zero vector is measured against 1e-3 of the largest norm (2)
    assert abs(s["max"] - 1e-6) < 1e-12
    assert s["median"] < 1e-6
    sc = run_configs.rel_stats(np.array([1.0, 2.0]), np.array([1.0, 1.0]))
    assert abs(sc["max"] - 1.0) < 1e-15
