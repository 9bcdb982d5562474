"""The smooth bound-mass functional of the step derivative: its hand-written
gradient (the seed of the backward pass) against central differences, and its
hard-threshold limit against the bound mass (e < 0 bound)."""
import numpy as np

from research_codes_gb300 import adjoint


def _state(n=40, seed=0):
    rng = np.random.default_rng(seed)
    return (rng.random(n) + 0.5, rng.normal(size=(n, 3)), -1.0 - rng.random(n), 0.3 * rng.random(n),
            rng.random(n) + 0.1)


def test_bound_mass_gradient_matches_central_differences():
    mass, vel, pot, uene, dens = _state()
    e0 = 0.7
    L, g = adjoint.bound_mass(mass, vel, pot, uene, dens, e0)
    eps = 1e-6
    for name, arr in (("vel", vel), ("pot", pot), ("uene", uene), ("dens", dens)):
        flat = arr.reshape(-1)
        for k in (0, 7, len(flat) - 1):
            keep = flat[k]
            flat[k] = keep + eps
            lp = adjoint.bound_mass(mass, vel, pot, uene, dens, e0)[0]
            flat[k] = keep - eps
            lm = adjoint.bound_mass(mass, vel, pot, uene, dens, e0)[0]
            flat[k] = keep
            fd = (lp - lm) / (2 * eps)
            ad = g[name].reshape(-1)[k]
            assert abs(ad - fd) <= 1e-6 * max(abs(fd), 1e-3), (name, k, ad, fd)


def test_bound_mass_hard_limit():
    """e0 -> 0 gives the bound mass of analysis/unbound_mass/unbound_mass.py:
    sum of m over particles with e < 0 (about the density-weighted velocity)."""
    mass, vel, pot, uene, dens = _state(seed=3)
    pot[:10] = 5.0   # some unbound particles
    vcm = (dens[:, None] * vel).sum(0) / dens.sum()
    e = 0.5 * ((vel - vcm) ** 2).sum(1) + pot + uene
    L, _ = adjoint.bound_mass(mass, vel, pot, uene, dens, 1e-9)
    assert np.isclose(L, mass[e < 0].sum(), rtol=1e-12)
