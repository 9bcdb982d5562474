"""Autotuner of the run parameters that shape the GPU work, not the physics.

Tuned by coordinate descent on the device time of a force evaluation of the
system's current state, as the captured steps run it: CUDA events of
replays of the captured force-evaluation graph (gravity lists on the second
stream, no host round trips), median of `reps`:

* n_group — the most i-particles a walk (i-group) may hold, which sets the
  list lengths and the pairs per step (the reference's FDPS setting is 256,
  main.cpp:380,386,394);
* item_split_nj — list length above which a walk's work items shrink to
  16, 8 or 4 i-particles, i.e. more lanes (threads) per i-particle, each
  taking a share of the j-tile stream;
* heavy_classes — how many of the most expensive work-item classes start
  first before the rest run in walk order;
* gravity_jtile — the j-tile of the gravity kernel: list entries a warp
  stages in shared memory and sums per pass (32 or 64).

Every candidate evaluates the same state, so the physics results differ only
through the list composition (pairs beyond the kernel support contribute
nothing; the signal-velocity maximum is taken over each walk's list, as in the
reference).
"""
import itertools

import numpy as np

CANDIDATES = {"n_group": (64, 80, 96, 128, 192, 256), "item_split_nj": (512, 1024, 2048, 4096, 8192, 1 << 30),
              "heavy_classes": (0, 1, 2, 4), "gravity_jtile": (32, 64)}


def time_forces(ps, reps=3):
    """Median device time (ms) of `reps` replays of the captured
    force-evaluation graph, after the evaluation that captures it."""
    ps.set_graph(True)
    ps.compute_forces()
    t = []
    for _ in range(reps):
        ps.compute_forces()
        t.append(ps.phase_times()["force_total"])
    return float(np.median(t))


def autotune(ps, candidates=None, reps=3, sweeps=2, apply=True):
    """Coordinate descent over the candidate values; returns (best parameter
    dict, list of (parameters, ms) tried).  The system keeps the best
    parameters when `apply` is set, else its original ones."""
    cand = dict(CANDIDATES if candidates is None else candidates)
    keys = list(cand)
    original = {k: getattr(ps.params, k) for k in keys}
    use_graph = ps.params.use_graph
    best = dict(original)
    tried = {}

    def measure(p):
        key = tuple(p[k] for k in keys)
        if key not in tried:
            ps.set_params(**p)
            tried[key] = time_forces(ps, reps)
        return tried[key]

    best_ms = measure(best)
    for _ in range(sweeps):
        improved = False
        for k in keys:
            for v in cand[k]:
                p = dict(best, **{k: v})
                ms = measure(p)
                if ms < best_ms:
                    best, best_ms, improved = p, ms, True
        if not improved:
            break
    ps.set_params(**(best if apply else original))
    # one evaluation with the kept parameters sizes the system's list and
    # task buffers for them before any graph is captured
    ps.compute_forces()
    ps.set_graph(bool(use_graph))
    table = [(dict(zip(keys, key)), ms) for key, ms in sorted(tried.items(), key=lambda kv: kv[1])]
    return best, table


def grid(candidates=None):
    """All combinations of the candidate values (for exhaustive searches)."""
    cand = CANDIDATES if candidates is None else candidates
    keys = list(cand)
    return [dict(zip(keys, v)) for v in itertools.product(*(cand[k] for k in keys))]
