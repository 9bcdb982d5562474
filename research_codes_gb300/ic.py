"""Synthetic initial conditions: Lane-Emden polytropes and two-star placement.

Restates the pipeline of the reference's polytropic_initial_condition tool
(main.cpp:12-227, lane_emden.hpp:14-53): a cubic lattice inside the unit
sphere is remapped radially so that each particle's enclosed-mass fraction
matches the Lane-Emden profile, then scaled to (M, R).  Differences, kept on
purpose:
  * the lattice gets a seeded random phase and rotation (the reference's is
    fixed), so that configurations are reproducible but not lattice-aligned;
  * the mass profile integrates rho = rho_c theta^n (the reference tool
    integrates theta itself, main.cpp:107-110);
  * u = n_eos P / rho with the code's ideal-gas closure n_eos = 1.5
    (hdr_hgas.hpp:339); the tool writes n P (main.cpp:225), a dimensional slip
    that the reference's relaxation overwrites.
All returned quantities are in code units (units.py).
"""
import math

import numpy as np

from . import units


def lane_emden(n, dr=1.0e-3, r0=1.0e-4):
    """RK4 solution of theta'' + 2/xi theta' + theta^n = 0 (lane_emden.hpp:14-53).

    Returns (xi, theta, dtheta) up to the first zero xi_1 (linearly located).
    """
    xi = r0
    th = 1.0 - r0 * r0 / 6.0 + n * r0 ** 4 / 120.0
    dth = -r0 / 3.0 + n * r0 ** 3 / 30.0

    def f(x, t, v):
        tn = t ** n if t > 0.0 else 0.0
        return v, -tn - 2.0 / x * v

    xs, ts, vs = [xi], [th], [dth]
    while True:
        k1 = f(xi, th, dth)
        k2 = f(xi + dr / 2, th + dr / 2 * k1[0], dth + dr / 2 * k1[1])
        k3 = f(xi + dr / 2, th + dr / 2 * k2[0], dth + dr / 2 * k2[1])
        k4 = f(xi + dr, th + dr * k3[0], dth + dr * k3[1])
        th_n = th + dr / 6 * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0])
        dth_n = dth + dr / 6 * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1])
        xi_n = xi + dr
        if th_n <= 0.0:
            frac = th / (th - th_n)
            xs.append(xi + frac * dr)
            ts.append(0.0)
            vs.append(dth + frac * (dth_n - dth))
            break
        xi, th, dth = xi_n, th_n, dth_n
        xs.append(xi)
        ts.append(th)
        vs.append(dth)
    return np.array(xs), np.array(ts), np.array(vs)


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def unit_lattice_sphere(n_target, rng):
    """Seeded random-phase, randomly rotated cubic lattice cut to r < 1."""
    s = (4.0 * math.pi / (3.0 * n_target)) ** (1.0 / 3.0)
    m = int(math.ceil(1.8 / s)) + 2
    g = (np.arange(-m, m + 1, dtype=np.float64)) * s
    phase = rng.uniform(0.0, s, size=3)
    x, y, z = np.meshgrid(g + phase[0], g + phase[1], g + phase[2], indexing="ij")
    p = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    p = p @ _random_rotation(rng).T
    r = np.sqrt((p * p).sum(1))
    p = p[r < 1.0]
    # trim or pad to exactly n_target by radius rank
    r = np.sqrt((p * p).sum(1))
    order = np.argsort(r, kind="stable")
    p = p[order]
    if len(p) >= n_target:
        p = p[:n_target]
    else:
        extra = rng.normal(size=(n_target - len(p), 3))
        extra /= np.linalg.norm(extra, axis=1, keepdims=True)
        extra *= rng.uniform(0.0, 1.0, size=(len(extra), 1)) ** (1.0 / 3.0)
        p = np.concatenate([p, extra])
    return p


def polytrope(n_part, mass_msun, radius_rsun, n_index, seed=0, eta=1.6):
    """One polytropic star centred on the origin at rest.

    Returns a dict of FP64 arrays in code units: pos (n,3), vel (n,3), mass,
    uene, ksr, dens (Lane-Emden density at each particle), plus scalars.
    """
    rng = np.random.default_rng(seed)
    xi, th, dth = lane_emden(n_index)
    xi1, dth1 = xi[-1], dth[-1]
    # enclosed-mass fraction m(xi)/M = xi^2 theta'(xi) / (xi1^2 theta'(xi1))
    mfrac = (xi * xi * dth) / (xi1 * xi1 * dth1)
    mfrac = np.maximum.accumulate(mfrac)

    p = unit_lattice_sphere(n_part, rng)
    r_u = np.sqrt((p * p).sum(1))
    order = np.argsort(r_u, kind="stable")
    f = np.empty(n_part)
    f[order] = (np.arange(n_part) + 0.5) / n_part
    xi_p = np.interp(f, mfrac, xi)

    M = mass_msun * units.SOLAR_MASS / units.UNIT_MASS
    R = radius_rsun * units.SOLAR_RADIUS / units.UNIT_LENGTH
    a = R / xi1
    rho_c = M / (4.0 * math.pi * a ** 3 * (-xi1 * xi1 * dth1))
    K = 4.0 * math.pi * units.G * a * a * rho_c ** (1.0 - 1.0 / n_index) / (n_index + 1.0)

    scale = np.where(r_u > 0, (xi_p * a) / np.maximum(r_u, 1e-300), 0.0)
    pos = p * scale[:, None]
    theta_p = np.interp(xi_p, xi, th)
    dens = rho_c * np.maximum(theta_p, 1e-6) ** n_index
    pres = K * dens ** (1.0 + 1.0 / n_index)
    mass = np.full(n_part, M / n_part)
    uene = units.EOS_N * pres / dens
    ksr = eta * units.KSRH * (mass / dens) ** (1.0 / 3.0)
    return dict(pos=pos, vel=np.zeros_like(pos), mass=mass, uene=uene, ksr=ksr, dens=dens,
                M=M, R=R, K=K, rho_c=rho_c)


def escape_speed(m_tot, separation):
    return math.sqrt(2.0 * units.G * m_tot / separation)


def two_stars(star1, star2, separation, impact, v_rel):
    """Places two stars in their centre-of-mass frame.

    Star 1 sits at -x, star 2 at +x, separated by `separation` along x and
    offset by `impact` along y; the relative velocity v_rel points along -x for
    star 2 (head-on when impact == 0).  Returns a dict with concatenated arrays
    and `istar` (0/1).
    """
    m1, m2 = star1["mass"].sum(), star2["mass"].sum()
    mt = m1 + m2
    d = np.array([separation, impact, 0.0])
    x1 = -d * m2 / mt
    x2 = d * m1 / mt
    v = np.array([-v_rel, 0.0, 0.0])
    v1 = -v * m2 / mt
    v2 = v * m1 / mt
    out = {}
    for key in ("mass", "uene", "ksr", "dens"):
        out[key] = np.concatenate([star1[key], star2[key]])
    out["pos"] = np.concatenate([star1["pos"] + x1, star2["pos"] + x2])
    out["vel"] = np.concatenate([star1["vel"] + v1, star2["vel"] + v2])
    out["istar"] = np.concatenate([np.zeros(len(star1["mass"]), np.int64),
                                   np.ones(len(star2["mass"]), np.int64)])
    return out


def config_system(name, scale=1.0, seed=0):
    """The particle systems of the five benchmark configurations.

    `scale` multiplies particle counts (tests use small scales).
    Returns (system dict, eta).
    """
    def n(k):
        return max(int(round(k * scale)), 64)

    if name == "c0":      # single n=1.5 polytrope, 1 Msun / 1 Rsun, ~50 neighbours
        eta = 1.18
        s = polytrope(n(10_000), 1.0, 1.0, 1.5, seed=seed, eta=eta)
        s["istar"] = np.zeros(len(s["mass"]), np.int64)
        return s, eta
    if name == "c1" or name == "c3":   # head-on, 2 x n=3 10 Msun / 4 Rsun
        eta = 1.18
        npart = 100_000 if name == "c1" else 50_000
        a = polytrope(n(npart), 10.0, 4.0, 3.0, seed=seed, eta=eta)
        b = polytrope(n(npart), 10.0, 4.0, 3.0, seed=seed + 1, eta=eta)
        R = a["R"]
        sep = 2.5 * R
        v = escape_speed(a["M"] + b["M"], sep)
        return two_stars(a, b, sep, 0.0, v), eta
    if name == "c2":      # off-axis unequal mass, N = 1M
        eta = 1.18
        a = polytrope(n(600_000), 10.0, 4.0, 3.0, seed=seed, eta=eta)
        b = polytrope(n(400_000), 3.0, 1.5, 1.5, seed=seed + 1, eta=eta)
        R1, R2 = a["R"], b["R"]
        sep = 3.0 * (R1 + R2)
        imp = 0.5 * (R1 + R2)
        v = 1.2 * escape_speed(a["M"] + b["M"], math.hypot(sep, imp))
        return two_stars(a, b, sep, imp, v), eta
    if name == "c4":      # N = 4M split 2:1, ~64 neighbours
        eta = 1.28
        a = polytrope(n(2_666_667), 10.0, 4.0, 3.0, seed=seed, eta=eta)
        b = polytrope(n(1_333_333), 5.0, 2.5, 3.0, seed=seed + 1, eta=eta)
        R1, R2 = a["R"], b["R"]
        sep = 3.0 * (R1 + R2)
        imp = 0.3 * (R1 + R2)
        v = escape_speed(a["M"] + b["M"], math.hypot(sep, imp))
        return two_stars(a, b, sep, imp, v), eta
    raise ValueError(name)
