"""The allocation-free gravity entry point (sph_calc_gravity_ep_noalloc).

Callers that cannot allocate device memory (host code that must not
synchronise the device, fixed-arena runtimes) pass device buffers they
already own; the entry point keeps its scratch in a static device array of
the library.  This test calls it through the C ABI with device buffers made
by torch (the test may allocate; the entry point does not), twice in a row
with different inputs, and compares each result with the existing
sph_calc_gravity_ep and with the FP64 oracle on the same inputs at the FP32C
tolerance used by the other GPU tests (1e-5 relative); once more at the size
limits (n_i = 4096, n_j = 65536); and checks that a call leaves the device's
free memory unchanged.

The file name sorts last so that a stop-at-first-failure run has executed
every other test before this one.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as orc
from research_codes_gb300 import _lib, abi, functors, walks

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _case(seed, n=2000, ni=150):
    rng = np.random.default_rng(seed)
    pos = rng.normal(size=(n, 3)) * 50.0 + 3.0e3       # far from the origin
    mass = rng.uniform(0.5, 1.5, n)
    h = rng.uniform(5.0, 10.0, n)
    s = dict(pos=pos, mass=mass, ksr=h)
    gi = np.arange(ni)
    return walks.gravity_epi(gi, s), walks.gravity_epj(np.arange(n), s)


def _entry():
    fn = _lib.load().sph_calc_gravity_ep_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                   ctypes.c_void_p]
    return fn


def _noalloc(epi, epj, force0, check_free=False):
    torch = pytest.importorskip("torch")
    fn = _entry()
    d_epi = torch.from_numpy(epi.view(np.uint8).copy()).cuda()
    d_epj = torch.from_numpy(epj.view(np.uint8).copy()).cuda()
    d_f = torch.from_numpy(force0.view(np.uint8).copy()).cuda()
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    st = fn(d_epi.data_ptr(), len(epi), d_epj.data_ptr(), len(epj), d_f.data_ptr(), stream.cuda_stream)
    assert st == abi.SPH_OK, abi.STATUS_NAMES.get(st, st)
    torch.cuda.synchronize()
    if check_free:
        # nothing allocated on the device by the call (after a first call has
        # loaded the library's module on this device)
        assert torch.cuda.mem_get_info()[0] == free0
    return d_f.cpu().numpy().view(abi.Gravity).copy()


def _oracle(epi, epj, force0):
    out = force0.copy()
    return orc.gravity(epi, epj, out=out)


def _existing(epi, epj, force0):
    out = force0.copy()
    with functors.Context(precision="fp32c") as ctx:
        functors.calcGravity(ctx)(epi, len(epi), epj, len(epj), out)
    return out


@pytest.mark.parametrize("call", [0])
def test_noalloc_matches_existing_entry_twice(call):
    for seed in (1, 2):                       # two calls in a row on the shared scratch
        epi, epj = _case(seed, ni=150 + 37 * seed)
        force0 = np.zeros(len(epi), abi.Gravity)
        force0["pot"] = -1.0 * seed           # accumulation semantics
        got = _noalloc(epi, epj, force0, check_free=seed == 2)
        ref = _existing(epi, epj, force0)
        exact = _oracle(epi, epj, force0)
        for f in ("acc", "pot", "eta"):
            assert rel_err(got[f], ref[f]).max() < TOL, (seed, f, rel_err(got[f], ref[f]).max())
            assert rel_err(got[f], exact[f]).max() < TOL, (seed, f, rel_err(got[f], exact[f]).max())


def test_noalloc_at_the_size_limits():
    """n_i = SPH_NOALLOC_MAX_I and n_j = SPH_NOALLOC_MAX_J: the whole scratch
    layout in use; against the FP64 oracle on a sample of i-particles."""
    n_i, n_j = 4096, 65536
    epi, epj = _case(3, n=n_j, ni=n_i)
    force0 = np.zeros(n_i, abi.Gravity)
    got = _noalloc(epi, epj, force0, check_free=True)
    sel = np.arange(0, n_i, 37)
    exact = _oracle(epi[sel], epj, force0[sel])
    for f in ("acc", "pot", "eta"):
        assert rel_err(got[f][sel], exact[f]).max() < TOL, (f, rel_err(got[f][sel], exact[f]).max())


def test_noalloc_rejects_oversized_calls():
    fn = _entry()
    assert fn(ctypes.c_void_p(16), 4097, ctypes.c_void_p(16), 10, ctypes.c_void_p(16), None) == abi.SPH_ERR_CAPACITY
    assert fn(ctypes.c_void_p(16), 10, ctypes.c_void_p(16), 65537, ctypes.c_void_p(16), None) == abi.SPH_ERR_CAPACITY
    assert fn(None, 10, None, 10, None, None) == abi.SPH_ERR_INVALID_ARGUMENT
