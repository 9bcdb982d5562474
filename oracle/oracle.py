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
REF_GLUE_SO = os.path.join(HERE, "_ref", "libsph_ref_glue.so")
# the reference's sph_yamauchi/run directory (only where the reference tree is)
REF_DIR = os.environ.get("SPH_REF_DIR")

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double


def build(ref=False):
    """make -C oracle [ref]; returns True when the requested libraries exist."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref and REF_DIR and os.path.isdir(REF_DIR):
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
        lib.oracle_sum_acceleration.argtypes = [ctypes.c_int64, _P, _P, _P, _P]
        lib.oracle_predict.argtypes = [ctypes.c_int64, _D] + [_P] * 13
        lib.oracle_correct.argtypes = [ctypes.c_int64, _D] + [_P] * 12
        lib.oracle_energy.argtypes = [ctypes.c_int64, _P, _P, _P, _P, _P]
        lib.oracle_energy.restype = _D
        lib.oracle_center_of_mass.argtypes = [ctypes.c_int64, _P, _P, _P, _P, ctypes.c_int32, _P]
        lib.oracle_ksrmax.argtypes = [ctypes.c_int64, _P, _P, _P, _P, _P]
        lib.oracle_ksrmax.restype = _D
        lib.oracle_timestep_pow2.argtypes = [_D, _D, _D, _D, _D]
        lib.oracle_timestep_pow2.restype = _D
        lib.oracle_gravity_lists.argtypes = [ctypes.c_int64, _P, _P, _P, _P, ctypes.c_int32, _P, _P, _D,
                                             ctypes.c_int32, _P, _P, _P, _P, _P, _P, _I]
        lib.oracle_gravity_lists.restype = ctypes.c_int64
        lib.oracle_neighbour_lists.argtypes = [ctypes.c_int64, _P, _P, _P, ctypes.c_int32, _P, _P, _P,
                                               ctypes.c_int32, ctypes.c_int32, _P, _P, _I]
        lib.oracle_neighbour_lists.restype = None
        _oracle = lib
    return _oracle


def ref_available(avx2=False):
    return os.path.exists(REF_AVX2_SO if avx2 else REF_SO)


def ref_glue_available():
    return os.path.exists(REF_GLUE_SO)


_ref_glue = None


def ref_glue_lib():
    """The reference's per-particle step glue (oracle/ref_glue.cpp)."""
    global _ref_glue
    if _ref_glue is None:
        lib = ctypes.CDLL(REF_GLUE_SO)
        n = ctypes.c_int64
        lib.ref_glue_eos.argtypes = [n] + [_P] * 4
        lib.ref_glue_balsara.argtypes = [n] + [_P] * 5
        lib.ref_glue_alpha_dot.argtypes = [n] + [_P] * 4 + [_D, _D, _P]
        lib.ref_glue_timestep.argtypes = [n] + [_P] * 5 + [_D, _D, _P]
        lib.ref_glue_energy.argtypes = [n] + [_P] * 5
        lib.ref_glue_predict.argtypes = [n, _D] + [_P] * 13
        lib.ref_glue_correct.argtypes = [n, _D] + [_P] * 12
        lib.ref_glue_sum_acceleration.argtypes = [n] + [_P] * 4
        lib.ref_glue_ksrmax.argtypes = [n] + [_P] * 5
        lib.ref_glue_ksrmax.restype = _D
        _ref_glue = lib
    return _ref_glue


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


def _f64(a):
    return np.ascontiguousarray(a, np.float64)


def sum_acceleration(acch, accg1, accg2):
    a, b, c = _f64(acch), _f64(accg1), _f64(accg2)
    out = np.empty_like(a)
    oracle_lib().oracle_sum_acceleration(len(a), _ptr(a), _ptr(b), _ptr(c), _ptr(out))
    return out


def predict(dt, s):
    """Leapfrog predictor on a copy of the state dict s (pos, vel, acc, uene,
    udot, alph, adot, alphu, adotu); returns the predicted dict with vel2,
    uene2, alph2, alphu2 added."""
    o = {k: _f64(s[k]).copy() for k in ("pos", "vel", "uene", "alph", "alphu")}
    acc, udot, adot, adotu = (_f64(s[k]) for k in ("acc", "udot", "adot", "adotu"))
    n = len(o["uene"])
    o["vel2"] = np.empty_like(o["vel"])
    for k in ("uene2", "alph2", "alphu2"):
        o[k] = np.empty(n)
    oracle_lib().oracle_predict(n, dt, _ptr(o["pos"]), _ptr(o["vel"]), _ptr(acc), _ptr(o["vel2"]),
                                _ptr(o["uene"]), _ptr(o["uene2"]), _ptr(udot), _ptr(o["alph"]),
                                _ptr(o["alph2"]), _ptr(adot), _ptr(o["alphu"]), _ptr(o["alphu2"]),
                                _ptr(adotu))
    return o


def correct(dt, s):
    """Leapfrog corrector: from the predicted half-step values (vel2, uene2,
    alph2, alphu2) and the new derivatives (acc, udot, adot, adotu) of dict s;
    returns vel, uene, alph, alphu."""
    vel2, uene2, alph2, alphu2 = (_f64(s[k]) for k in ("vel2", "uene2", "alph2", "alphu2"))
    acc, udot, adot, adotu = (_f64(s[k]) for k in ("acc", "udot", "adot", "adotu"))
    n = len(uene2)
    o = {"vel": np.empty_like(vel2), "uene": np.empty(n), "alph": np.empty(n), "alphu": np.empty(n)}
    oracle_lib().oracle_correct(n, dt, _ptr(o["vel"]), _ptr(vel2), _ptr(acc), _ptr(o["uene"]), _ptr(uene2),
                                _ptr(udot), _ptr(o["alph"]), _ptr(alph2), _ptr(adot), _ptr(o["alphu"]),
                                _ptr(alphu2), _ptr(adotu))
    return o


def energy(mass, vel, uene, pot):
    """(total, kinetic, thermal, potential)."""
    arrs = [_f64(a) for a in (mass, vel, uene, pot)]
    parts = np.zeros(3)
    e = oracle_lib().oracle_energy(len(arrs[0]), *[_ptr(a) for a in arrs], _ptr(parts))
    return (e, *parts)


def center_of_mass(mass, pos, vel, istar, star=-1):
    m, p, v = _f64(mass), _f64(pos), _f64(vel)
    st = np.ascontiguousarray(istar, np.int32)
    out = np.zeros(7)
    oracle_lib().oracle_center_of_mass(len(m), _ptr(m), _ptr(p), _ptr(v), _ptr(st), star, _ptr(out))
    return out


def ksrmax(mass, pos, vel, istar, dens):
    m, p, v, d = _f64(mass), _f64(pos), _f64(vel), _f64(dens)
    st = np.ascontiguousarray(istar, np.int32)
    return oracle_lib().oracle_ksrmax(len(m), _ptr(m), _ptr(p), _ptr(v), _ptr(st), _ptr(d))


def timestep_pow2(dt, dtc, time, dt_max, dt_min):
    return oracle_lib().oracle_timestep_pow2(dt, dtc, time, dt_max, dt_min)


def alpha_dot(divv, alph, alphu, vsnd, ksr, uene, diffu, alpha_max, alpha_min, alphu_max, alphu_min, eps_u):
    """(adot, adotu) of calcAlphaDot (hdr_hgas.hpp:750-762), umin = 0."""
    arrs = [_f64(a) for a in (divv, alph, alphu, vsnd, ksr, uene, diffu)]
    n = len(arrs[0])
    adot, adotu = np.empty(n), np.empty(n)
    oracle_lib().oracle_alpha_dot(n, *[_ptr(a) for a in arrs], alpha_max, alpha_min, alphu_max, alphu_min, eps_u,
                                  _ptr(adot), _ptr(adotu))
    return adot, adotu


def timestep_min(ksr, vsmx, divv, accg, c_dt, dt_max):
    """Minimum over dt_max and the particles' limits (hdr_hgas.hpp:477-488);
    accg = a_g1 + a_g2 (n x 3)."""
    k, v, d, g = _f64(ksr), _f64(vsmx), _f64(divv), _f64(accg)
    return oracle_lib().oracle_timestep_min(len(k), _ptr(k), _ptr(v), _ptr(d), _ptr(g), c_dt, dt_max)


def gravity_tree_lists(keys, pos, mass, eps2, gfirst, gcount, theta=0.5, n_leaf=8, nthreads=0):
    """Host octree walk (oracle_gravity_lists): per group the particle entries
    (ep_off, ep_idx) and accepted nodes (sp_off, sp_idx), with the nodes'
    monopoles (x, y, z, mass) and mass-weighted eps^2.  keys must be sorted
    and pos, mass, eps2 in that order."""
    lib = oracle_lib()
    keys = np.ascontiguousarray(keys, np.uint64)
    pos, mass, eps2 = _f64(pos), _f64(mass), _f64(eps2)
    gfirst = np.ascontiguousarray(gfirst, np.int64)
    gcount = np.ascontiguousarray(gcount, np.int64)
    ng = len(gfirst)
    ep_off = np.zeros(ng + 1, np.int64)
    sp_off = np.zeros(ng + 1, np.int64)
    args = (len(mass), _ptr(keys), _ptr(pos), _ptr(mass), _ptr(eps2), ng, _ptr(gfirst), _ptr(gcount), theta,
            n_leaf, _ptr(ep_off), _ptr(sp_off))
    nn = lib.oracle_gravity_lists(*args, None, None, None, None, nthreads)
    ep_idx = np.zeros(max(int(ep_off[-1]), 1), np.int32)
    sp_idx = np.zeros(max(int(sp_off[-1]), 1), np.int32)
    mom = np.zeros((nn, 4))
    neps2 = np.zeros(nn)
    lib.oracle_gravity_lists(*args, _ptr(ep_idx), _ptr(sp_idx), _ptr(mom), _ptr(neps2), nthreads)
    return ep_off, ep_idx, sp_off, sp_idx, mom, neps2


def neighbour_lists(keys, pos, h, gfirst, gcount, gr, mode, n_leaf=8, nthreads=0):
    """Host octree neighbour lists (oracle_neighbour_lists): per group g the
    particles within gr[g] of its bounding box (mode 0, gather) or within
    max(gr[g], h_j) (mode 1, symmetric), ascending; gr < 0 gives an empty
    list.  Returns (off, idx).  keys must be sorted, pos and h in that order."""
    lib = oracle_lib()
    keys = np.ascontiguousarray(keys, np.uint64)
    pos, h, gr = _f64(pos), _f64(h), _f64(gr)
    gfirst = np.ascontiguousarray(gfirst, np.int64)
    gcount = np.ascontiguousarray(gcount, np.int64)
    ng = len(gfirst)
    off = np.zeros(ng + 1, np.int64)
    args = (len(h), _ptr(keys), _ptr(pos), _ptr(h), ng, _ptr(gfirst), _ptr(gcount), _ptr(gr), int(mode), n_leaf,
            _ptr(off))
    lib.oracle_neighbour_lists(*args, None, nthreads)
    idx = np.zeros(max(int(off[-1]), 1), np.int32)
    lib.oracle_neighbour_lists(*args, _ptr(idx), nthreads)
    return off, idx[:int(off[-1])]
