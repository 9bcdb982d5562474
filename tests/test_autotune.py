"""CPU tests of the autotuner's search (coordinate descent, caching, restoring
the system's parameters) against a fake system whose force-evaluation time is
a known function of the parameters."""
import types

from research_codes_gb300 import autotune


class FakeSystem:
    def __init__(self, cost, **params):
        self.params = types.SimpleNamespace(use_graph=1, **params)
        self.cost = cost
        self.evaluations = 0
        self.graph_calls = []

    def set_params(self, **kw):
        for k, v in kw.items():
            setattr(self.params, k, v)

    def set_graph(self, on):
        self.graph_calls.append(bool(on))
        self.params.use_graph = int(bool(on))

    def compute_forces(self):
        self.evaluations += 1

    def phase_times(self):
        p = self.params
        return {"force_total": self.cost(p.n_group, p.item_split_nj, p.heavy_classes, p.gravity_jtile)}


START = dict(n_group=256, item_split_nj=1 << 30, heavy_classes=0, gravity_jtile=32)


def _separable(g, s, h, jt):
    return 1.0 + abs(g - 128) / 64 + abs(s - 4096) / 4096 + 0.1 * abs(h - 2) + (0.05 if jt == 32 else 0.0)


def test_coordinate_descent_finds_the_minimum_of_a_separable_cost():
    ps = FakeSystem(_separable, **START)
    best, table = autotune.autotune(ps, reps=3)
    assert best == dict(n_group=128, item_split_nj=4096, heavy_classes=2, gravity_jtile=64)
    # the system keeps the best parameters and its graph setting
    assert {k: getattr(ps.params, k) for k in best} == best
    assert ps.params.use_graph == 1 and ps.graph_calls[-1] is True
    # the table is sorted by time, every combination measured once
    ms = [t for _, t in table]
    assert ms == sorted(ms) and table[0][0] == best and abs(ms[0] - 1.0) < 1e-12
    keys = [tuple(sorted(p.items())) for p, _ in table]
    assert len(keys) == len(set(keys))
    # one warm-up plus `reps` evaluations per distinct combination
    assert ps.evaluations == 4 * len(table) + 1   # and one with the kept parameters


def test_apply_false_restores_the_original_parameters():
    ps = FakeSystem(_separable, **START)
    best, _ = autotune.autotune(ps, reps=1, apply=False)
    assert best != START
    assert {k: getattr(ps.params, k) for k in START} == START


def test_result_is_a_coordinate_minimum_of_a_coupled_cost():
    # n_group and item_split_nj interact: the best split depends on the group size
    def coupled(g, s, h, jt):
        return 1.0 + ((g / 128.0) * (s / 4096.0) - 1.0) ** 2 + abs(g - 256) / 1024 + 0.01 * h + 0.001 * jt
    ps = FakeSystem(coupled, **START)
    best, table = autotune.autotune(ps, reps=1, sweeps=3)
    t_best = coupled(*best.values())
    assert t_best <= coupled(*START.values())
    for k, vals in autotune.CANDIDATES.items():
        for v in vals:
            p = dict(best, **{k: v})
            assert coupled(p["n_group"], p["item_split_nj"], p["heavy_classes"], p["gravity_jtile"]) >= t_best


def test_grid_enumerates_every_combination():
    g = autotune.grid({"a": (1, 2), "b": (3, 4, 5)})
    assert len(g) == 6 and {"a": 2, "b": 5} in g
    assert len(autotune.grid()) == 6 * 6 * 4 * 2


def test_candidates_are_valid_system_parameters():
    # the values sph_system_set_params accepts (include/sph_gb300.h):
    # n_group >= 1, gravity_jtile 32 or 64; item_split_nj <= 0 means the
    # default, so every candidate split is a positive length
    c = autotune.CANDIDATES
    assert set(c) == {"n_group", "item_split_nj", "heavy_classes", "gravity_jtile"}
    assert all(isinstance(v, int) and v >= 1 for v in c["n_group"])
    assert all(isinstance(v, int) and v > 0 for v in c["item_split_nj"])
    assert all(isinstance(v, int) and v >= 0 for v in c["heavy_classes"])
    assert set(c["gravity_jtile"]) <= {32, 64}
    # the reference's own group size stays among the candidates (main.cpp:380)
    assert 256 in c["n_group"]
