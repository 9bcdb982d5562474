import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "functors_n1000.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


def rel_err(a, b, floor_frac=1e-6):
    """Elementwise |a-b| / max(|b|, floor_frac * max|b|) over the last axis norm.

    For vector fields (…,3) the norm of the difference is divided by the norm
    of the reference vector, floored at floor_frac times the field's largest
    norm so that near-zero vectors (symmetric neighbourhoods) do not dominate.
    """
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.ndim > 1:
        d = np.linalg.norm(a - b, axis=-1)
        s = np.linalg.norm(b, axis=-1)
    else:
        d = np.abs(a - b)
        s = np.abs(b)
    floor = floor_frac * (s.max() if s.size else 0.0)
    return d / np.maximum(s, max(floor, 1e-300))


def walk_slices(i_off, j_off):
    for w in range(len(i_off) - 1):
        yield w, slice(int(i_off[w]), int(i_off[w + 1])), slice(int(j_off[w]), int(j_off[w + 1]))


def field_errors(a, b, floor_frac=1e-3):
    """Summary of per-particle relative errors (floored as rel_err) plus the
    normwise error ||a-b|| / ||b|| over the whole field."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    r = rel_err(a, b, floor_frac)
    return {"max": float(r.max()), "p999": float(np.quantile(r, 0.999)), "median": float(np.median(r)),
            "normwise": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))}


def assert_cancelling_field(a, b, name, floor_frac=1e-3):
    """Acceptance for sums that cancel strongly (the SPH pressure gradient,
    du/dt and softening correction of a star near hydrostatic equilibrium,
    where the pair terms are ~R/h times larger than their sum) computed by
    two engines from inputs that differ at rounding level: the median and the
    normwise difference within 1e-5, the 99.9th percentile within 1e-4."""
    e = field_errors(a, b, floor_frac)
    assert e["median"] < 1e-5 and e["normwise"] < 1e-5 and e["p999"] < 1e-4, (name, e)
