"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE).

Two libraries:
  * ``oracle/liboracle.so``      — the C restatement (sph_oracle.c), built on
    any host by ``make -C oracle``;
  * ``oracle/_ref/libsph_ref.so`` — the reference's own functors compiled from
    the reference source tree (``make -C oracle ref``); present only where
    that tree is.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module.
"""
import ctypes
import os
import subprocess

import numpy as np

from research_codes_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsph_ref.so")
REF_AVX2_SO = os.path.join(HERE, "_ref", "libsph_ref_avx2.so")
REF_DIR = os.environ.get("SPH_REF_DIR", "/root/reference/sph_yamauchi/run")

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double


def build(ref=False):
    """make -C oracle [ref]; returns True when the requested libraries exist."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref and os.path.isdir(REF_DIR):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={REF_DIR}"], check=True)
    return os.path.exists(ORACLE_SO) and (not ref or os.path.exists(REF_SO))


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class _Lib:
    def __init__(self, path, prefix):
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix

    def fn(self, name):
        return getattr(self.lib, self.prefix + name)


_oracle = None
_ref = {}


def oracle_lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            build()
        lib = ctypes.CDLL(ORACLE_SO)
        lib.oracle_density.argtypes = [_P, _I, _P, _I, _P, _D, _D]
        lib.oracle_hydro.argtypes = [_P, _I, _P, _I, _P]
        lib.oracle_gravity_ep.argtypes = [_P, _I, _P, _I, _P]
        lib.oracle_gravity_sp.argtypes = [_P, _I, _P, _I, _P]
        lib.oracle_density_walks.argtypes = [_I, _P, _P, _P, _P, _P, _D, _D, _I]
        lib.oracle_hydro_walks.argtypes = [_I, _P, _P, _P, _P, _P, _I]
        lib.oracle_gravity_walks.argtypes = [_I, _P, _P, _P, _P, _P, _I]
        for f in ("oracle_density_walks", "oracle_hydro_walks", "oracle_gravity_walks"):
            getattr(lib, f).restype = _I
        lib.oracle_eos.argtypes = [ctypes.c_int64, _P, _P, _P, _P]
        lib.oracle_balsara.argtypes = [ctypes.c_int64, _P, _P, _P, _P, _P]
        lib.oracle_alpha_dot.argtypes = [ctypes.c_int64] + [_P] * 7 + [_D] * 5 + [_P, _P]
        lib.oracle_timestep_min.argtypes = [ctypes.c_int64, _P, _P, _P, _P, _D, _D]
        lib.oracle_timestep_min.restype = _D
        _oracle = lib
    return _oracle


def ref_available(avx2=False):
    return os.path.exists(REF_AVX2_SO if avx2 else REF_SO)


def ref_lib(avx2=False):
    path = REF_AVX2_SO if avx2 else REF_SO
    if path not in _ref:
        lib = ctypes.CDLL(path)
        lib.ref_calc_density.argtypes = [_P, _I, _P, _I, _P, _D]
        lib.ref_calc_hydro.argtypes = [_P, _I, _P, _I, _P]
        lib.ref_calc_gravity_ep.argtypes = [_P, _I, _P, _I, _P]
        lib.ref_calc_gravity_sp.argtypes = [_P, _I, _P, _I, _P]
        lib.ref_density_walks.argtypes = [_I, _P, _P, _P, _P, _P, _D, _I]
        lib.ref_hydro_walks.argtypes = [_I, _P, _P, _P, _P, _P, _I]
        lib.ref_gravity_walks.argtypes = [_I, _P, _P, _P, _P, _P, _I]
        for f in ("ref_density_walks", "ref_hydro_walks", "ref_gravity_walks"):
            getattr(lib, f).restype = _I
        lib.ref_eta.restype = _D
        _ref[path] = lib
    return _ref[path]


# ---- single-group calls (numpy structured arrays in, new array out) --------

def density(epi, epj, eta=1.6, ksr_max=0.0, impl="oracle"):
    out = np.zeros(len(epi), abi.Density)
    epi = np.ascontiguousarray(epi, abi.DensityEPI)
    epj = np.ascontiguousarray(epj, abi.DensityEPJ)
    if impl == "oracle":
        oracle_lib().oracle_density(_ptr(epi), len(epi), _ptr(epj), len(epj), _ptr(out),
                                    eta, ksr_max)
    else:
        lib = ref_lib(impl == "ref_avx2")
        if abs(eta - lib.ref_eta()) > 0:
            raise ValueError("the reference's eta is a compile-time 1.6")
        lib.ref_calc_density(_ptr(epi), len(epi), _ptr(epj), len(epj), _ptr(out), ksr_max)
    return out


def hydro(epi, epj, impl="oracle"):
    out = np.zeros(len(epi), abi.Hydro)
    epi = np.ascontiguousarray(epi, abi.HydroEPI)
    epj = np.ascontiguousarray(epj, abi.HydroEPJ)
    if impl == "oracle":
        oracle_lib().oracle_hydro(_ptr(epi), len(epi), _ptr(epj), len(epj), _ptr(out))
    else:
        ref_lib(impl == "ref_avx2").ref_calc_hydro(_ptr(epi), len(epi), _ptr(epj), len(epj),
                                                   _ptr(out))
    return out


def gravity(epi, epj, spj=None, impl="oracle", out=None):
    """EPJ pass then SPJ pass, accumulating like FDPS's two functor calls."""
    if out is None:
        out = np.zeros(len(epi), abi.Gravity)
    epi = np.ascontiguousarray(epi, abi.GravityEPI)
    epj = np.ascontiguousarray(epj, abi.GravityEPJ)
    if impl == "oracle":
        lib = oracle_lib()
        lib.oracle_gravity_ep(_ptr(epi), len(epi), _ptr(epj), len(epj), _ptr(out))
        if spj is not None and len(spj):
            spj = np.ascontiguousarray(spj, abi.GravitySPJ)
            lib.oracle_gravity_sp(_ptr(epi), len(epi), _ptr(spj), len(spj), _ptr(out))
    else:
        lib = ref_lib(impl == "ref_avx2")
        lib.ref_calc_gravity_ep(_ptr(epi), len(epi), _ptr(epj), len(epj), _ptr(out))
        if spj is not None and len(spj):
            spj = np.ascontiguousarray(spj, abi.GravitySPJ)
            lib.ref_calc_gravity_sp(_ptr(epi), len(epi), _ptr(spj), len(spj), _ptr(out))
    return out


# ---- walk-batched calls -----------------------------------------------------

def density_walks(i_off, j_off, epi, epj, eta=1.6, ksr_max=0.0, nthreads=0, impl="oracle"):
    out = np.zeros(len(epi), abi.Density)
    i_off = np.ascontiguousarray(i_off, np.int64)
    j_off = np.ascontiguousarray(j_off, np.int64)
    nw = len(i_off) - 1
    if impl == "oracle":
        nt = oracle_lib().oracle_density_walks(nw, _ptr(i_off), _ptr(j_off), _ptr(epi),
                                               _ptr(epj), _ptr(out), eta, ksr_max, nthreads)
    else:
        nt = ref_lib(impl == "ref_avx2").ref_density_walks(
            nw, _ptr(i_off), _ptr(j_off), _ptr(epi), _ptr(epj), _ptr(out), ksr_max, nthreads)
    return out, nt


def hydro_walks(i_off, j_off, epi, epj, nthreads=0, impl="oracle"):
    out = np.zeros(len(epi), abi.Hydro)
    i_off = np.ascontiguousarray(i_off, np.int64)
    j_off = np.ascontiguousarray(j_off, np.int64)
    nw = len(i_off) - 1
    if impl == "oracle":
        nt = oracle_lib().oracle_hydro_walks(nw, _ptr(i_off), _ptr(j_off), _ptr(epi),
                                             _ptr(epj), _ptr(out), nthreads)
    else:
        nt = ref_lib(impl == "ref_avx2").ref_hydro_walks(
            nw, _ptr(i_off), _ptr(j_off), _ptr(epi), _ptr(epj), _ptr(out), nthreads)
    return out, nt


def gravity_walks(i_off, j_off, epi, epj, nthreads=0, impl="oracle"):
    out = np.zeros(len(epi), abi.Gravity)
    i_off = np.ascontiguousarray(i_off, np.int64)
    j_off = np.ascontiguousarray(j_off, np.int64)
    nw = len(i_off) - 1
    if impl == "oracle":
        nt = oracle_lib().oracle_gravity_walks(nw, _ptr(i_off), _ptr(j_off), _ptr(epi),
                                               _ptr(epj), _ptr(out), nthreads)
    else:
        nt = ref_lib(impl == "ref_avx2").ref_gravity_walks(
            nw, _ptr(i_off), _ptr(j_off), _ptr(epi), _ptr(epj), _ptr(out), nthreads)
    return out, nt


# ---- step glue ----------------------------------------------------------------

def eos(dens, uene):
    dens = np.ascontiguousarray(dens, np.float64)
    uene = np.ascontiguousarray(uene, np.float64)
    pres = np.empty_like(dens)
    vsnd = np.empty_like(dens)
    oracle_lib().oracle_eos(len(dens), _ptr(dens), _ptr(uene), _ptr(pres), _ptr(vsnd))
    return pres, vsnd


def balsara(divv, rotv, vsnd, ksr):
    arrs = [np.ascontiguousarray(a, np.float64) for a in (divv, rotv, vsnd, ksr)]
    out = np.empty_like(arrs[0])
    oracle_lib().oracle_balsara(len(out), *[_ptr(a) for a in arrs], _ptr(out))
    return out
