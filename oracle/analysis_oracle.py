"""Test infrastructure only: a numpy restatement of the reference's analysis
scripts, the oracle for research_codes_gb300.analysis.  Pinned against the
reference's own functions by tests/golden/analysis_n2000.npz.

  centre_of_gravity  analysis/common.py:71-90
  bound_mass         analysis/unbound_mass/unbound_mass.py:10-27
  lagrange_radii     analysis/lagrange_radius/lagrange_radius.py:25-47, 90-96
  orbit_energy       energy_check/energy_check.py:28-77
  energy_error       energy_check/energy_check.py:86-107
"""
import math

import numpy as np


def centre_of_gravity(pos, vel, dens):
    w = float(np.sum(dens))
    return (np.sum(dens[:, None] * pos, axis=0) / w, np.sum(dens[:, None] * vel, axis=0) / w)


def bound_mass(vel, pot, uene, mass, vel_ref):
    dv = vel - vel_ref
    e = 0.5 * np.sum(dv * dv, axis=1) + pot + uene
    unbound = float(np.sum(mass[e > 0.0]))
    return float(np.sum(mass)) - unbound, unbound


def lagrange_radii(pos, mass, centre, fractions=np.arange(1, 10) * 0.1):
    d = pos - centre
    r = np.sqrt(np.sum(d * d, axis=1))
    order = np.argsort(r, kind="stable")
    r, m = r[order], mass[order]
    total = float(np.sum(mass))
    targets = [total * f for f in fractions]
    cum, out, j = 0.0, [], 0
    for i in range(len(r)):
        cum += m[i]
        if cum > targets[j]:
            out.append(r[i - 1])
            j += 1
        if j == len(targets):
            break
    return np.array(out)


def orbit_energy(pos, vel, dens, mass, star, r1, r2, G):
    c = [centre_of_gravity(pos[star == s], vel[star == s], dens[star == s]) for s in (0, 1)]
    m = []
    for s, (x, _), R in zip((0, 1), c, (r1, r2)):
        d = pos[star == s] - x
        m.append(float(np.sum(mass[star == s][np.sqrt(np.sum(d * d, axis=1)) < 2 * R])))
    ke = 0.5 * m[0] * float(c[0][1] @ c[0][1]) + 0.5 * m[1] * float(c[1][1] @ c[1][1])
    d = c[0][0] - c[1][0]
    return ke - G * m[0] * m[1] / math.sqrt(float(d @ d))


def energy_error(series, max_time):
    """(max error, its time, error at the end, end time) of (time, energy) rows."""
    e0 = series[0, 1]
    emax, tmax, eend, tend = 0.0, 0.0, 0.0, 0.0
    for t, e in series:
        if t >= max_time:
            eend, tend = e - e0, t
            if abs(eend) >= abs(emax):
                emax, tmax = eend, t
            break
        if abs(e - e0) > abs(emax):
            emax, tmax = e - e0, t
    return emax, tmax, eend, tend
