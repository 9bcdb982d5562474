"""Analysis of a run's state on the device: the reference's post-processing
scripts, computed from the engine's FP64 state without writing snapshots.

* centre_of_gravity — density-weighted centre and velocity
  (analysis/common.py:71-90)
* bound_mass — bound / unbound mass about a reference velocity
  (analysis/unbound_mass/unbound_mass.py:10-27, 50-58)
* lagrange_radii — radii enclosing 10 %, ..., 90 % of the mass about the
  density-weighted centre (analysis/lagrange_radius/lagrange_radius.py:25-47,
  73-96)
* binary_orbit_energy — orbital energy of two stars as point masses
  (energy_check/energy_check.py:28-77)

Particle sets: all particles (star=None) or one star (istar == star).
Reductions, distances and the distance sort run on the device; the
cumulative mass of the Lagrange radii is taken on the host in the sorted
order, as the reference accumulates it.
"""
import ctypes

import numpy as np

from . import _lib
from .abi import SPHError

_D = ctypes.c_double
_P = ctypes.c_void_p


def _lib_decl():
    lib = _lib.load()
    sig = {"sph_system_center_of_gravity": [_P, ctypes.c_int32, _P],
           "sph_system_bound_mass": [_P, ctypes.c_int32, _P, _P],
           "sph_system_mass_within": [_P, ctypes.c_int32, _P, _D, _P],
           "sph_system_radii_sorted": [_P, ctypes.c_int32, _P, _P, _P, _P]}
    for name, args in sig.items():
        f = getattr(lib, name)
        f.restype = ctypes.c_int
        f.argtypes = args
    return lib


def _arr(x):
    a = np.ascontiguousarray(x, dtype=np.float64)
    return a, a.ctypes.data_as(_P)


def _star(star):
    return -1 if star is None else int(star)


def _check(ps, st, what):
    if st:
        buf = ctypes.create_string_buffer(512)
        _lib.load().sph_context_last_error(ps.ctx.handle, buf, 512)
        raise SPHError(st, f"{what}: {buf.value.decode(errors='replace')}")


def centre_of_gravity(ps, star=None):
    """(position[3], velocity[3]) weighted by density."""
    out, po = _arr(np.zeros(7))
    _check(ps, _lib_decl().sph_system_center_of_gravity(ps.handle, _star(star), po), "centre_of_gravity")
    return out[:3].copy(), out[3:6].copy()


def bound_mass(ps, star=None, vel_ref=None):
    """(bound, unbound) mass of the set; the reference velocity defaults to
    the set's density-weighted velocity."""
    if vel_ref is None:
        vel_ref = centre_of_gravity(ps, star)[1]
    v, pv = _arr(vel_ref)
    out, po = _arr(np.zeros(2))
    _check(ps, _lib_decl().sph_system_bound_mass(ps.handle, _star(star), pv, po), "bound_mass")
    return float(out[0]), float(out[1])


def mass_within(ps, center, radius, star=None):
    c, pc = _arr(center)
    out, po = _arr(np.zeros(1))
    _check(ps, _lib_decl().sph_system_mass_within(ps.handle, _star(star), pc, float(radius), po), "mass_within")
    return float(out[0])


def radii_sorted(ps, center, star=None):
    """Distances from `center` of the set's particles in ascending order, with
    their masses."""
    c, pc = _arr(center)
    r = np.empty(ps.n)
    m = np.empty(ps.n)
    cnt = ctypes.c_int64(0)
    _check(ps, _lib_decl().sph_system_radii_sorted(ps.handle, _star(star), pc, r.ctypes.data_as(_P),
                                                    m.ctypes.data_as(_P), ctypes.byref(cnt)), "radii_sorted")
    return r[:cnt.value], m[:cnt.value]


def lagrange_from_sorted(r, m, mass_total=None, fractions=np.arange(1, 10) * 0.1):
    """The reference's rule on radii sorted ascending: walking outwards, the
    first particle whose cumulative mass exceeds fraction_j of the total
    records the radius of the particle before it; one fraction per particle."""
    if mass_total is None:
        mass_total = float(np.sum(m))
    targets = [mass_total * f for f in fractions]
    cum = np.cumsum(m)
    out, j = [], 0
    for i in range(len(r)):
        if j == len(targets):
            break
        if cum[i] > targets[j]:
            out.append(float(r[i - 1]))
            j += 1
    return np.array(out)


def lagrange_radii(ps, star=None, center=None, fractions=np.arange(1, 10) * 0.1):
    """Radii enclosing the given mass fractions about the set's
    density-weighted centre (or `center`)."""
    if center is None:
        center = centre_of_gravity(ps, star)[0]
    r, m = radii_sorted(ps, center, star)
    return lagrange_from_sorted(r, m, fractions=fractions)


def binary_orbit_energy(ps, r1, r2, G):
    """Kinetic + potential energy of the two stars (istar 0 and 1) as point
    masses: each star's mass within twice its radius of its density-weighted
    centre, moving with its density-weighted velocity."""
    (x0, v0), (x1, v1) = centre_of_gravity(ps, 0), centre_of_gravity(ps, 1)
    m0 = mass_within(ps, x0, 2.0 * r1, 0)
    m1 = mass_within(ps, x1, 2.0 * r2, 1)
    ke = 0.5 * m0 * float(v0 @ v0) + 0.5 * m1 * float(v1 @ v1)
    d = x0 - x1
    return ke - G * m0 * m1 / float(np.sqrt(d @ d))


def energy_error(times, energies, max_time=None):
    """The reference's energy check of a run's energy record
    (energy_check/energy_check.py:86-107): (largest |E - E0| up to max_time
    with its sign and time, E - E0 at max_time and that time)."""
    t = np.asarray(times, dtype=np.float64)
    e = np.asarray(energies, dtype=np.float64)
    if max_time is None:
        max_time = float(t[-1])
    e0 = e[0]
    emax, tmax, eend, tend = 0.0, 0.0, 0.0, 0.0
    for ti, ei in zip(t, e):
        if ti >= max_time:
            eend, tend = ei - e0, ti
            if abs(eend) >= abs(emax):
                emax, tmax = eend, ti
            break
        if abs(ei - e0) > abs(emax):
            emax, tmax = ei - e0, ti
    return float(emax), float(tmax), float(eend), float(tend)
