"""C ABI checks that need no GPU: the library builds and loads, exports every
function include/sph_gb300.h declares, and its struct layouts equal both the
numpy mirrors and the reference classes' sizes."""
import ctypes
import os

import pytest

from research_codes_gb300 import _lib, abi


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def test_exports_every_header_function(lib):
    names = _lib.header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_layout_matches_numpy_mirrors(lib):
    n = lib.sph_abi_layout(None, 0)
    buf = (ctypes.c_int64 * n)()
    assert lib.sph_abi_layout(buf, n) == n
    assert list(buf) == abi.layout_vector()
    for name, dt in abi.LAYOUT_ORDER:
        assert dt.itemsize == abi.EXPECTED_SIZES[name], name


def test_status_strings(lib):
    assert lib.sph_status_string(0) == b"ok"
    assert b"capacity" in lib.sph_status_string(abi.SPH_ERR_CAPACITY)
    assert lib.sph_version().startswith(b"sph_gb300")


def test_params_default(lib):
    p = _lib.Params()
    lib.sph_params_default(ctypes.byref(p))
    assert (p.eta, p.max_walks, p.max_i, p.max_j) == (1.6, 1000, 1_000_000, 10_000_000)


def test_invalid_arguments_rejected_without_device(lib):
    h = ctypes.c_void_p()
    p = _lib.Params()
    lib.sph_params_default(ctypes.byref(p))
    p.eta = -1.0
    assert lib.sph_context_create(ctypes.byref(p), ctypes.byref(h)) == abi.SPH_ERR_INVALID_ARGUMENT
    assert lib.sph_context_create(ctypes.byref(p), None) == abi.SPH_ERR_INVALID_ARGUMENT
    assert lib.sph_context_destroy(None) == abi.SPH_ERR_INVALID_ARGUMENT
    assert lib.sph_calc_density(None, None, 0, None, 0, None) == abi.SPH_ERR_INVALID_ARGUMENT


def test_no_device_is_reported_cleanly(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert lib.sph_context_create(None, ctypes.byref(h)) == abi.SPH_ERR_NO_DEVICE
    assert not h.value


def test_c_struct_mirrors_match_the_header(tmp_path):
    """sizeof and every member offset of the parameter and statistics structs,
    compiled from include/sph_gb300.h by the host C compiler, equal the ctypes
    mirrors the Python layer reads them with."""
    import shutil
    import subprocess

    from research_codes_gb300 import system
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    mirrors = [("sph_params", _lib.Params), ("sph_system_params", system.SystemParams),
               ("sph_system_stats", system.SystemStats)]
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "sph_gb300.h"', "int main(void) {"]
    for cname, cls in mirrors:
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("%zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c11", f"-I{inc}", str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    want = []
    for _, cls in mirrors:
        want.append(ctypes.sizeof(cls))
        want += [getattr(cls, f).offset for f, _ in cls._fields_]
    assert got == want


def test_time_step_limits_are_validated_before_any_device_call():
    """dt_min <= 0 or an infinite dt_max would let the step-halving loop run
    without end; sph_system_create rejects them before it touches the
    context, so a zeroed stand-in context suffices here."""
    from research_codes_gb300 import system
    lib = system._declare(_lib.load())
    fake_ctx = ctypes.create_string_buffer(1 << 16)
    out = ctypes.c_void_p()
    for dt_min, dt_max in ((0.0, 10.0), (-1e-16, 10.0), (1e-16, float("inf")), (1.0, 0.5),
                           (float("nan"), 10.0)):
        p = system.SystemParams()
        lib.sph_system_params_default(ctypes.byref(p))
        p.dt_min, p.dt_max = dt_min, dt_max
        assert lib.sph_system_create(ctypes.cast(fake_ctx, ctypes.c_void_p), 1000, ctypes.byref(p),
                                     ctypes.byref(out)) == abi.SPH_ERR_INVALID_ARGUMENT, (dt_min, dt_max)
        assert not out.value
