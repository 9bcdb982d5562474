"""Python mirror of the reference's interaction-functor interface.

The reference hands FDPS three functors, calcDensity (hdr_density.hpp:246),
calcHydro (hdr_hydro.hpp:312) and calcGravity<TJ> (hdr_gravity.hpp:286), called
as ``functor(epi, n_i, epj, n_j, force)``, and on GPUs the multiwalk pairs
DispatchKernel_* / RetrieveKernel_* (use_gpu.hpp:28-64).  The classes and
functions below keep those names, argument orders and meanings; arrays are
numpy structured arrays with the dtypes of ``abi``.  Every call runs on the
GPU through libsph_gb300.so.

Differences from the reference, by design:
  * a Context (device, precision, eta, ksrmax, capacities) is passed
    explicitly instead of file-static device buffers and RP:: globals;
  * failures raise abi.SPHError instead of assert()/silent corruption.
"""
import ctypes
import weakref

import numpy as np

from . import abi
from ._lib import Params, check, load

_PREC = {"fp32c": abi.PREC_FP32C, "fp64": abi.PREC_FP64,
         abi.PREC_FP32C: abi.PREC_FP32C, abi.PREC_FP64: abi.PREC_FP64}


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and len(a) else ctypes.c_void_p(0)


def _require(a, dtype, name):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous numpy array of dtype abi.{name}")


class Context:
    """One GPU context: a CUDA stream plus device buffers (sph_context)."""

    def __init__(self, device=0, precision="fp32c", eta=1.6, ksr_max=0.0, max_walks=1000,
                 max_i=1_000_000, max_j=10_000_000, check_finite=True):
        lib = load()
        p = Params()
        lib.sph_params_default(ctypes.byref(p))
        p.device = device
        p.precision = _PREC[precision]
        p.eta = eta
        p.ksr_max = ksr_max
        p.max_walks = max_walks
        p.max_i = int(max_i)
        p.max_j = int(max_j)
        p.check_finite = 1 if check_finite else 0
        h = ctypes.c_void_p()
        check(lib.sph_context_create(ctypes.byref(p), ctypes.byref(h)), what="sph_context_create")
        self.handle = h
        self.lib = lib
        self._systems = weakref.WeakSet()

    def close(self):
        if getattr(self, "handle", None):
            # systems on this context go first (they use its stream)
            for sys_ in list(getattr(self, "_systems", ())):
                sys_.close()
            self.lib.sph_context_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_eta(self, eta):
        check(self.lib.sph_context_set_eta(self.handle, eta), self.handle)

    def set_ksr_max(self, ksr_max):
        check(self.lib.sph_context_set_ksr_max(self.handle, ksr_max), self.handle)

    def set_precision(self, precision):
        check(self.lib.sph_context_set_precision(self.handle, _PREC[precision]), self.handle)

    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        p = ctypes.c_void_p()
        check(self.lib.sph_context_stream(self.handle, ctypes.byref(p)), self.handle)
        return p.value or 0

    def probe_fp32_peak(self):
        """Measured FP32 FMA throughput of the device, TFLOP/s."""
        v = ctypes.c_double()
        check(self.lib.sph_probe_fp32_peak(self.handle, ctypes.byref(v)), self.handle, "probe")
        return v.value


class calcDensity:
    """calcDensity::operator() (hdr_density.hpp:248-252); assigns force[:n_i]."""

    def __init__(self, ctx):
        self.ctx = ctx

    def __call__(self, epi, nip, epj, njp, density):
        _require(epi, abi.DensityEPI, "DensityEPI")
        _require(epj, abi.DensityEPJ, "DensityEPJ")
        _require(density, abi.Density, "Density")
        if nip > len(epi) or njp > len(epj) or nip > len(density):
            raise ValueError("counts exceed array lengths")
        c = self.ctx
        check(c.lib.sph_calc_density(c.handle, _ptr(epi), nip, _ptr(epj), njp, _ptr(density)),
              c.handle, "calcDensity")


class calcHydro:
    """calcHydro::operator() (hdr_hydro.hpp:314-318); assigns force[:n_i]."""

    def __init__(self, ctx):
        self.ctx = ctx

    def __call__(self, epi, nip, epj, njp, hydro):
        _require(epi, abi.HydroEPI, "HydroEPI")
        _require(epj, abi.HydroEPJ, "HydroEPJ")
        _require(hydro, abi.Hydro, "Hydro")
        if nip > len(epi) or njp > len(epj) or nip > len(hydro):
            raise ValueError("counts exceed array lengths")
        c = self.ctx
        check(c.lib.sph_calc_hydro(c.handle, _ptr(epi), nip, _ptr(epj), njp, _ptr(hydro)),
              c.handle, "calcHydro")


class calcGravity:
    """calcGravity<TJ>::operator() (hdr_gravity.hpp:289-293).

    TJ is chosen by the dtype of the j array (GravityEPJ or GravitySPJ).
    ACCUMULATES into force[:n_i], like the reference."""

    def __init__(self, ctx):
        self.ctx = ctx

    def __call__(self, epi, nip, epj, njp, gravity):
        _require(epi, abi.GravityEPI, "GravityEPI")
        _require(gravity, abi.Gravity, "Gravity")
        if epj.dtype == abi.GravityEPJ and epj.dtype.names == abi.GravityEPJ.names:
            fn = self.ctx.lib.sph_calc_gravity_ep
        else:
            _require(epj, abi.GravitySPJ, "GravitySPJ")
            fn = self.ctx.lib.sph_calc_gravity_sp
        if nip > len(epi) or njp > len(epj) or nip > len(gravity):
            raise ValueError("counts exceed array lengths")
        c = self.ctx
        check(fn(c.handle, _ptr(epi), nip, _ptr(epj), njp, _ptr(gravity)), c.handle, "calcGravity")


# ---- multiwalk Dispatch / Retrieve -------------------------------------------

def _ptr_array(arrs):
    return (ctypes.c_void_p * max(len(arrs), 1))(*[a.ctypes.data if len(a) else 0 for a in arrs])


def _count_array(counts):
    return (ctypes.c_int32 * max(len(counts), 1))(*[int(c) for c in counts])


def DispatchKernel_Dens(ctx, tag, n_walk, epi, n_epi, epj, n_epj):
    """DispatchKernel_Dens (hdr_densityGPU.cu:496-592): epi/epj are lists of arrays."""
    check(ctx.lib.sph_dispatch_density(ctx.handle, tag, n_walk, _ptr_array(epi), _count_array(n_epi),
                                       _ptr_array(epj), _count_array(n_epj)), ctx.handle, "dispatch")
    ctx._keep = (epi, epj)
    return 0


def RetrieveKernel_Dens(ctx, tag, n_walk, ni, density):
    """RetrieveKernel_Dens (hdr_densityGPU.cu:594-621): fills the arrays of `density`."""
    check(ctx.lib.sph_retrieve_density(ctx.handle, tag, n_walk, _count_array(ni), _ptr_array(density)),
          ctx.handle, "retrieve")
    return 0


def DispatchKernel_HydroForce(ctx, tag, n_walk, epi, n_epi, epj, n_epj):
    """DispatchKernel_HydroForce (hdr_hydroGPU.cu:371-476)."""
    check(ctx.lib.sph_dispatch_hydro(ctx.handle, tag, n_walk, _ptr_array(epi), _count_array(n_epi),
                                     _ptr_array(epj), _count_array(n_epj)), ctx.handle, "dispatch")
    ctx._keep = (epi, epj)
    return 0


def RetrieveKernel_HydroForce(ctx, tag, n_walk, ni, hydro):
    """RetrieveKernel_HydroForce (hdr_hydroGPU.cu:478-507)."""
    check(ctx.lib.sph_retrieve_hydro(ctx.handle, tag, n_walk, _count_array(ni), _ptr_array(hydro)),
          ctx.handle, "retrieve")
    return 0


def DispatchKernel_Gravity(ctx, tag, n_walk, epi, n_epi, epj, n_epj, spj, n_spj):
    """DispatchKernel_Gravity (hdr_gravityGPU.cu:383-469)."""
    check(ctx.lib.sph_dispatch_gravity(ctx.handle, tag, n_walk, _ptr_array(epi), _count_array(n_epi),
                                       _ptr_array(epj), _count_array(n_epj), _ptr_array(spj),
                                       _count_array(n_spj)), ctx.handle, "dispatch")
    ctx._keep = (epi, epj, spj)
    return 0


def RetrieveKernel_Gravity(ctx, tag, n_walk, ni, gravity):
    """RetrieveKernel_Gravity (hdr_gravityGPU.cu:471-495); assigns the totals."""
    check(ctx.lib.sph_retrieve_gravity(ctx.handle, tag, n_walk, _count_array(ni), _ptr_array(gravity)),
          ctx.handle, "retrieve")
    return 0
