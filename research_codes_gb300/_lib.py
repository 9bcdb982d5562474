"""ctypes binding of libsph_gb300.so (include/sph_gb300.h).

The library is the only compute path: when it is missing or fails to load,
every call raises; there is no CPU fallback.
"""
import ctypes
import os
import re

from . import abi
from .build import INCLUDE, LIB

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double
_PP = ctypes.POINTER(ctypes.c_void_p)
_PI32 = ctypes.POINTER(ctypes.c_int32)


class Params(ctypes.Structure):
    """struct sph_params."""
    _fields_ = [("device", _I32), ("precision", _I32), ("eta", _D), ("ksr_max", _D),
                ("max_walks", _I32), ("max_i", _I64), ("max_j", _I64), ("check_finite", _I32)]


_lib = None


def header_functions():
    """Names of all functions declared in include/sph_gb300.h."""
    text = open(os.path.join(INCLUDE, "sph_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sph_[a-z0-9_]+)\s*\(", text)))


def _declare(lib):
    sig = {
        "sph_params_default": (None, [ctypes.POINTER(Params)]),
        "sph_context_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(_P)]),
        "sph_context_destroy": (ctypes.c_int, [_P]),
        "sph_context_set_eta": (ctypes.c_int, [_P, _D]),
        "sph_context_set_ksr_max": (ctypes.c_int, [_P, _D]),
        "sph_context_set_precision": (ctypes.c_int, [_P, _I32]),
        "sph_status_string": (ctypes.c_char_p, [ctypes.c_int]),
        "sph_context_last_error": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
        "sph_calc_density": (ctypes.c_int, [_P, _P, _I32, _P, _I32, _P]),
        "sph_calc_hydro": (ctypes.c_int, [_P, _P, _I32, _P, _I32, _P]),
        "sph_calc_gravity_ep": (ctypes.c_int, [_P, _P, _I32, _P, _I32, _P]),
        "sph_calc_gravity_sp": (ctypes.c_int, [_P, _P, _I32, _P, _I32, _P]),
        "sph_dispatch_density": (ctypes.c_int, [_P, _I32, _I32, _PP, _PI32, _PP, _PI32]),
        "sph_retrieve_density": (ctypes.c_int, [_P, _I32, _I32, _PI32, _PP]),
        "sph_dispatch_hydro": (ctypes.c_int, [_P, _I32, _I32, _PP, _PI32, _PP, _PI32]),
        "sph_retrieve_hydro": (ctypes.c_int, [_P, _I32, _I32, _PI32, _PP]),
        "sph_dispatch_gravity": (ctypes.c_int, [_P, _I32, _I32, _PP, _PI32, _PP, _PI32, _PP, _PI32]),
        "sph_retrieve_gravity": (ctypes.c_int, [_P, _I32, _I32, _PI32, _PP]),
        "sph_abi_layout": (_I64, [ctypes.POINTER(_I64), _I64]),
        "sph_version": (ctypes.c_char_p, []),
        "sph_context_stream": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
        "sph_probe_fp32_peak": (ctypes.c_int, [_P, ctypes.POINTER(_D)]),
    }
    for name, (res, args) in sig.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
    return lib


def load(build_if_missing=True):
    """Loads (building first when absent) and returns the ctypes library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        if not build_if_missing:
            raise RuntimeError(f"{LIB} is missing: run research_codes_gb300.build.build()")
        from .build import build
        build()
    _lib = _declare(ctypes.CDLL(LIB))
    return _lib


def check(status, ctx=None, what=""):
    if status == abi.SPH_OK:
        return
    detail = what
    if ctx is not None:
        buf = ctypes.create_string_buffer(512)
        load().sph_context_last_error(ctx, buf, 512)
        detail = f"{what}: {buf.value.decode(errors='replace')}" if what else buf.value.decode(errors="replace")
    raise abi.SPHError(status, detail)
