"""Device-resident particle system (sph_system_* in include/sph_gb300.h).

    with functors.Context(precision="fp32c", eta=1.18) as ctx:
        sys = ParticleSystem(ctx, n)
        sys.upload(state)             # dict of numpy arrays (ic.polytrope & co.)
        sys.compute_forces()          # calcSPHKernel, main.cpp:300-358
        sys.step(10)                  # loopSimulation body, hdr_hgas.hpp:1499-1540
        acc = sys.download("acc")

The whole step runs on the GPU: the tree and interaction lists that FDPS
provides to the reference are built by the engine itself.
"""
import ctypes

import numpy as np

from . import units
from ._lib import check, load

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double

FIELDS = {"pos": (0, 3), "vel": (1, 3), "acc": (2, 3), "acch": (3, 3), "accg1": (4, 3), "accg2": (5, 3),
          "mass": (10, 1), "dens": (11, 1), "pres": (12, 1), "vsnd": (13, 1), "ksr": (14, 1),
          "divv": (15, 1), "rotv": (16, 1), "bswt": (17, 1), "grdh": (18, 1), "uene": (19, 1),
          "udot": (20, 1), "alph": (21, 1), "alphu": (22, 1), "pot": (23, 1), "eta": (24, 1),
          "vsmx": (25, 1), "diffu": (26, 1), "np": (27, 1), "adot": (28, 1), "adotu": (29, 1),
          "id": (30, 1), "istar": (31, 1)}


class SystemParams(ctypes.Structure):
    _fields_ = [("n_group", _I32), ("n_leaf", _I32), ("theta", _D), ("G", _D), ("c_dt", _D),
                ("dt_max", _D), ("dt_min", _D), ("alpha_max", _D), ("alpha_min", _D),
                ("alphu_max", _D), ("alphu_min", _D), ("ksr_max_mode", _I32),
                ("max_density_iterations", _I32), ("use_graph", _I32), ("quadrupole", _I32),
                ("item_split_nj", _I32), ("heavy_classes", _I32), ("density_list_slack", ctypes.c_float),
                ("hydro_signal_skip", _I32), ("gravity_jtile", _I32)]


class SystemStats(ctypes.Structure):
    _fields_ = [("time", _D), ("dt", _D), ("ksr_max", _D), ("e_kin", _D), ("e_thm", _D), ("e_pot", _D),
                ("e_tot", _D), ("n_groups", _I64), ("density_iterations", _I64), ("pairs_density", _I64),
                ("pairs_density_first", _I64), ("pairs_hydro", _I64), ("pairs_gravity", _I64), ("list_density", _I64),
                ("list_hydro", _I64), ("list_gravity", _I64), ("steps", _I64), ("density_rechecked", _I64),
                ("evals_density_first", _I64), ("evals_density_grad", _I64), ("evals_hydro_near", _I64),
                ("evals_hydro_far", _I64), ("density_list_passes", _I64),
                ("density_sweep_passes", _I64), ("hydro_sv_tiles_skipped", _I64), ("hydro_sv_tiles", _I64),
                ("hydro_pairs_marked", _I64), ("hydro_pair_slots", _I64), ("hydro_rows_overflowed", _I64),
                ("last_status", _I32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _declare(lib):
    sig = {
        "sph_system_params_default": (None, [ctypes.POINTER(SystemParams)]),
        "sph_system_create": (ctypes.c_int, [_P, _I64, ctypes.POINTER(SystemParams), ctypes.POINTER(_P)]),
        "sph_system_destroy": (ctypes.c_int, [_P]),
        "sph_system_upload": (ctypes.c_int, [_P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
        "sph_system_compute_forces": (ctypes.c_int, [_P]),
        "sph_system_step": (ctypes.c_int, [_P, _I32]),
        "sph_system_download": (ctypes.c_int, [_P, _I32, _P]),
        "sph_system_download_sorted": (ctypes.c_int, [_P, _I32, _P]),
        "sph_system_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(SystemStats)]),
        "sph_system_get_lists": (ctypes.c_int, [_P, _I32, ctypes.POINTER(_I32), ctypes.POINTER(_I64),
                                                _P, _P, _P, _P]),
        "sph_system_get_nodes": (ctypes.c_int, [_P, _P, _P]),
        "sph_system_phase_times": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float), _I32]),
        "sph_system_set_graph": (ctypes.c_int, [_P, _I32]),
        "sph_system_graph_kernels": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.c_int64)]),
        "sph_system_set_field": (ctypes.c_int, [_P, _I32, _P]),
        "sph_system_set_params": (ctypes.c_int, [_P, ctypes.POINTER(SystemParams)]),
        "sph_system_get_clock": (ctypes.c_int, [_P, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(_D),
                                                ctypes.POINTER(_D)]),
        "sph_system_set_clock": (ctypes.c_int, [_P, _D, _D, _D, _D]),
        "sph_system_predict": (ctypes.c_int, [_P]),
        "sph_system_adjoint_forces": (ctypes.c_int, [_P, _P, _P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def default_params(**kw):
    lib = _declare(load())
    p = SystemParams()
    lib.sph_system_params_default(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


class ParticleSystem:
    def __init__(self, ctx, n, **params):
        self.lib = _declare(load())
        self.ctx = ctx
        self.n = int(n)
        self.params = default_params(**params)
        h = ctypes.c_void_p()
        check(self.lib.sph_system_create(ctx.handle, self.n, ctypes.byref(self.params), ctypes.byref(h)),
              ctx.handle, "sph_system_create")
        self.handle = h
        if hasattr(ctx, "_systems"):
            ctx._systems.add(self)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.sph_system_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, s, t0=0.0):
        n = self.n
        c = lambda k, dt=np.float64: np.ascontiguousarray(s[k], dt)  # noqa: E731
        ids = c("id", np.int64) if "id" in s else np.arange(n, dtype=np.int64)
        istar = c("istar", np.int32) if "istar" in s else None
        alph = c("alph") if "alph" in s else None
        alphu = c("alphu") if "alphu" in s else None
        arrs = dict(ids=ids, istar=istar, mass=c("mass"), pos=c("pos"), vel=c("vel"), uene=c("uene"),
                    ksr=c("ksr"), alph=alph, alphu=alphu)
        for k, v in arrs.items():
            if v is not None and len(v) != n:
                raise ValueError(f"{k} has {len(v)} entries, system has {n}")
        self._keep = arrs
        check(self.lib.sph_system_upload(self.handle, t0, _ptr(ids), _ptr(istar), _ptr(arrs["mass"]),
                                         _ptr(arrs["pos"]), _ptr(arrs["vel"]), _ptr(arrs["uene"]),
                                         _ptr(arrs["ksr"]), _ptr(alph), _ptr(alphu)),
              self.ctx.handle, "upload")

    def compute_forces(self):
        check(self.lib.sph_system_compute_forces(self.handle), self.ctx.handle, "compute_forces")

    def predict(self):
        """Leapfrog predictor alone, with the clock's dt."""
        check(self.lib.sph_system_predict(self.handle), self.ctx.handle, "predict")

    SEED = (("acc", 3), ("udot", 1), ("adot", 1), ("ksr", 1), ("pot", 1), ("dens", 1))
    GRAD = (("pos", 3), ("vel", 3), ("uene", 1), ("alph", 1), ("ksr", 1))

    def adjoint_forces(self, seed):
        """Vector-Jacobian product of the last force evaluation: `seed` maps
        output names (acc, udot, adot, ksr, pot, dens; missing ones are zero)
        to dL/d output in upload order; returns dL/d input for pos, vel, uene,
        alph and ksr (the evaluation's first guess of h)."""
        n = self.n
        buf = np.zeros(8 * n, np.float64)
        o = 0
        for k, w in self.SEED:
            if k in seed:
                buf[o:o + w * n] = np.asarray(seed[k], np.float64).reshape(-1)
            o += w * n
        out = np.empty(9 * n, np.float64)
        check(self.lib.sph_system_adjoint_forces(self.handle, _ptr(buf), _ptr(out)), self.ctx.handle,
              "adjoint_forces")
        res, o = {}, 0
        for k, w in self.GRAD:
            res[k] = out[o:o + w * n].reshape((n, 3) if w == 3 else n).copy()
            o += w * n
        return res

    def set_graph(self, on):
        check(self.lib.sph_system_set_graph(self.handle, 1 if on else 0), self.ctx.handle, "set_graph")

    def set_params(self, **params):
        """Changes run parameters (n_group, theta, item_split_nj, ...)."""
        for k, v in params.items():
            if k not in dict(SystemParams._fields_):
                raise KeyError(k)
            setattr(self.params, k, v)
        check(self.lib.sph_system_set_params(self.handle, ctypes.byref(self.params)), self.ctx.handle, "set_params")

    def set_field(self, field, data):
        """Host -> device copy of one field in upload order (restart)."""
        code, w = FIELDS[field]
        arr = np.ascontiguousarray(data, dtype=np.float64)
        if arr.size != self.n * w:
            raise ValueError(f"{field}: expected {self.n * w} values, got {arr.size}")
        check(self.lib.sph_system_set_field(self.handle, code, _ptr(arr)), self.ctx.handle, f"set_field {field}")

    def clock(self):
        """(time, dt, ksr_max, eps_u) of the run."""
        v = [_D() for _ in range(4)]
        check(self.lib.sph_system_get_clock(self.handle, *[ctypes.byref(x) for x in v]), self.ctx.handle, "clock")
        return tuple(x.value for x in v)

    def set_clock(self, time=-1.0, dt=-1.0, ksr_max=-1.0, eps_u=-1.0):
        check(self.lib.sph_system_set_clock(self.handle, time, dt, ksr_max, eps_u), self.ctx.handle, "set_clock")

    def graph_kernels(self, step=True):
        """Kernel launches per replay of the captured step (or force) graph."""
        k = ctypes.c_int64(0)
        check(self.lib.sph_system_graph_kernels(self.handle, 1 if step else 0, ctypes.byref(k)),
              self.ctx.handle, "graph_kernels")
        return int(k.value)

    def step(self, n_steps=1):
        check(self.lib.sph_system_step(self.handle, n_steps), self.ctx.handle, "step")

    def download(self, field, sorted_order=False, out=None):
        code, w = FIELDS[field]
        if out is None:
            out = np.empty((self.n, 3) if w == 3 else self.n, np.float64)
        fn = self.lib.sph_system_download_sorted if sorted_order else self.lib.sph_system_download
        check(fn(self.handle, code, _ptr(out)), self.ctx.handle, f"download {field}")
        return out

    def stats(self):
        st = SystemStats()
        check(self.lib.sph_system_get_stats(self.handle, ctypes.byref(st)), self.ctx.handle, "stats")
        return st.as_dict()

    def lists(self, kind):
        """(i_first, i_count, j_off, j_idx) of the last evaluation; kind 0/1/2 =
        density / hydro / gravity, 3 = the last density re-walk (its groups;
        it evaluates their still-iterating particles), in the system's sorted
        order."""
        nw = _I32()
        ne = _I64()
        check(self.lib.sph_system_get_lists(self.handle, kind, ctypes.byref(nw), ctypes.byref(ne),
                                            None, None, None, None), self.ctx.handle, "lists")
        i_first = np.empty(max(nw.value, 1), np.int32)
        i_count = np.empty(max(nw.value, 1), np.int32)
        j_off = np.empty(nw.value + 1, np.int64)
        j_idx = np.empty(max(ne.value, 1), np.int32)
        check(self.lib.sph_system_get_lists(self.handle, kind, ctypes.byref(nw), ctypes.byref(ne),
                                            _ptr(i_first), _ptr(i_count), _ptr(j_off), _ptr(j_idx)),
              self.ctx.handle, "lists")
        return i_first[:nw.value], i_count[:nw.value], j_off, j_idx[:ne.value]

    PHASES = ("tree", "density", "density_kernel", "gravity_lists", "gravity_kernel", "hydro_lists",
              "hydro_kernel", "force_total", "hydro_signal", "hydro_df")

    def phase_times(self):
        """Device ms of the phases of the last force evaluation (CUDA events)."""
        buf = (ctypes.c_float * 10)()
        k = self.lib.sph_system_phase_times(self.handle, buf, 10)
        if k < 0:
            check(-k, self.ctx.handle, "phase_times")
        return {name: float(buf[i]) for i, name in enumerate(self.PHASES[:k])}

    def nodes(self):
        mom = np.empty((2 * self.n - 1, 4), np.float64)
        eps2 = np.empty(2 * self.n - 1, np.float64)
        check(self.lib.sph_system_get_nodes(self.handle, _ptr(mom), _ptr(eps2)), self.ctx.handle, "nodes")
        return mom, eps2


def state_from_ic(s):
    """Adds the fields the engine needs to an ic.* dict (ids, alpha = 1, alphu = 0)."""
    n = len(s["mass"])
    out = dict(s)
    out.setdefault("id", np.arange(n, dtype=np.int64))
    out.setdefault("istar", np.zeros(n, np.int64))
    out.setdefault("alph", np.ones(n))
    out.setdefault("alphu", np.zeros(n))
    return out


G = units.G
