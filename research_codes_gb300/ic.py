"""Synthetic initial conditions: Lane-Emden polytropes, rescaled stars and
two-star placement (fixed separation and velocity, or an unbound Kepler orbit).

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


def polytrope_scalings(n_index, M, R, G):
    """Lane-Emden solution and the scalings of a polytrope of mass M and
    radius R (any consistent units): (xi, theta, theta', a = R / xi_1,
    rho_c, K) with rho = rho_c theta^n, r = a xi and P = K rho^(1 + 1/n)
    (the tool's convert_real_quantities, polytropic_initial_condition/
    main.cpp:205-227, with the first zero xi_1 located exactly)."""
    xi, th, dth = lane_emden(n_index)
    xi1, dth1 = xi[-1], dth[-1]
    a = R / xi1
    rho_c = M / (4.0 * math.pi * a ** 3 * (-xi1 * xi1 * dth1))
    K = 4.0 * math.pi * G * a * a * rho_c ** (1.0 - 1.0 / n_index) / (n_index + 1.0)
    return xi, th, dth, a, rho_c, K


def polytrope(n_part, mass_msun, radius_rsun, n_index, seed=0, eta=1.6):
    """One polytropic star centred on the origin at rest.

    Returns a dict of FP64 arrays in code units: pos (n,3), vel (n,3), mass,
    uene, ksr, dens (Lane-Emden density at each particle), plus the scalars
    M, R, K, rho_c and n_index.
    """
    rng = np.random.default_rng(seed)
    M = mass_msun * units.SOLAR_MASS / units.UNIT_MASS
    R = radius_rsun * units.SOLAR_RADIUS / units.UNIT_LENGTH
    xi, th, dth, a, rho_c, K = polytrope_scalings(n_index, M, R, units.G)
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

    scale = np.where(r_u > 0, (xi_p * a) / np.maximum(r_u, 1e-300), 0.0)
    pos = p * scale[:, None]
    theta_p = np.interp(xi_p, xi, th)
    dens = rho_c * np.maximum(theta_p, 1e-6) ** n_index
    pres = K * dens ** (1.0 + 1.0 / n_index)
    mass = np.full(n_part, M / n_part)
    uene = units.EOS_N * pres / dens
    ksr = eta * units.KSRH * (mass / dens) ** (1.0 / 3.0)
    return dict(pos=pos, vel=np.zeros_like(pos), mass=mass, uene=uene, ksr=ksr, dens=dens,
                M=M, R=R, K=K, rho_c=rho_c, n_index=n_index)


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


def rescale(star, m_mul, r_mul):
    """A relaxed star moved to mass x m_mul and radius x r_mul, as the
    reference's change_polytropic_scale tool does (main.cpp:96-115, factors
    user_define.hpp:9-10): positions and smoothing lengths scale with r_mul,
    velocities with sqrt(m_mul / r_mul), specific energies with
    m_mul / r_mul, which keeps the star in the same (scaled) equilibrium.
    Unit-independent: works on code-unit or cgs arrays alike.  Density-like
    extras (dens, rho_c, K) are scaled to stay consistent; the reference tool
    leaves its density column as read, since the run recomputes it."""
    v_mul = math.sqrt(m_mul / r_mul)
    u_mul = m_mul / r_mul
    out = dict(star)
    out["mass"] = star["mass"] * m_mul
    out["pos"] = star["pos"] * r_mul
    out["vel"] = star["vel"] * v_mul
    out["uene"] = star["uene"] * u_mul
    out["ksr"] = star["ksr"] * r_mul
    if "dens" in star:
        out["dens"] = star["dens"] * (m_mul / r_mul ** 3)
    if "M" in star:
        out["M"] = star["M"] * m_mul
    if "R" in star:
        out["R"] = star["R"] * r_mul
    if "rho_c" in star:
        out["rho_c"] = star["rho_c"] * (m_mul / r_mul ** 3)
    if "K" in star and "n_index" in star:
        n = star["n_index"]
        out["K"] = star["K"] * u_mul * (m_mul / r_mul ** 3) ** (-1.0 / n)
    return out


def unbound_orbit(m1, m2, r_peri, v_inf, r_sep, G=None):
    """Two point masses on the Kepler orbit with relative speed `v_inf` at
    infinity and pericentre distance `r_peri`, at separation `r_sep` before
    pericentre, in their centre-of-mass frame; the orbital plane is z = 0 and
    pericentre lies on +x.

    The reference's two_body_initial_condition tool (main.cpp:87-140, inputs
    user_define.hpp:13-24) derives the hyperbola from the impact parameter
    b = r_p v_p / v_inf and the energy k = v_inf^2 / 2: eccentricity
    e = sqrt(1 + 2 k (b v_inf)^2 / mu^2), true anomaly from
    r = a (e^2 - 1) / (1 + e cos f) with sin f < 0, and velocity
    sqrt(mu / p) (-sin f, e + cos f).  Here the same conic is written with
    the angular momentum h = r_p v_p and the semi-latus rectum
    p = h^2 / mu = r_p (1 + e), so that v_inf = 0 (the parabola, e = 1,
    p = 2 r_p) is the same formula.  Star 1 sits at m2 / M of the relative
    vector (star 1 minus star 2), star 2 at -m1 / M of it.

    Returns (x1, x2, v1, v2, elements) with 3-vectors and
    elements = {b, e, p, h, f}; raises ValueError when r_sep < r_peri.
    """
    if G is None:
        G = units.G
    if v_inf < 0 or r_peri <= 0:
        raise ValueError("need v_inf >= 0 and r_peri > 0")
    if r_sep < r_peri:
        raise ValueError("the stars start inside the pericentre distance")
    mu = G * (m1 + m2)
    k_inf = 0.5 * v_inf * v_inf
    v_p = math.sqrt(2.0 * (k_inf + mu / r_peri))
    h = r_peri * v_p
    e = math.sqrt(1.0 + 2.0 * k_inf * h * h / (mu * mu))
    p = h * h / mu
    cos_f = min(1.0, (p / r_sep - 1.0) / e)
    sin_f = -math.sqrt(max(0.0, 1.0 - cos_f * cos_f))
    w = math.sqrt(mu / p)
    rel_x = np.array([r_sep * cos_f, r_sep * sin_f, 0.0])
    rel_v = np.array([-w * sin_f, w * (cos_f + e), 0.0])
    q1, q2 = m2 / (m1 + m2), -m1 / (m1 + m2)
    el = {"b": h / v_inf if v_inf > 0 else math.inf, "e": e, "p": p, "h": h,
          "f": math.atan2(sin_f, cos_f)}
    return q1 * rel_x, q2 * rel_x, q1 * rel_v, q2 * rel_v, el


def two_stars_on_orbit(star1, star2, r_peri, v_inf, r_sep, G=None):
    """Places two stars on the orbit of `unbound_orbit` (the reference's
    two_body_initial_condition tool, main.cpp:142-158): each star's particles
    are shifted by its centre's position and velocity.  Returns the same
    layout as `two_stars`, plus `id` (star 2 numbered after star 1, as
    main.cpp:152 does) and the orbit's elements under `orbit`."""
    m1, m2 = star1["mass"].sum(), star2["mass"].sum()
    x1, x2, v1, v2, el = unbound_orbit(m1, m2, r_peri, v_inf, r_sep, G)
    n1, n2 = len(star1["mass"]), len(star2["mass"])
    out = {}
    for key in ("mass", "uene", "ksr", "dens"):
        if key in star1 and key in star2:
            out[key] = np.concatenate([star1[key], star2[key]])
    out["pos"] = np.concatenate([star1["pos"] + x1, star2["pos"] + x2])
    out["vel"] = np.concatenate([star1["vel"] + v1, star2["vel"] + v2])
    out["istar"] = np.concatenate([np.zeros(n1, np.int64), np.ones(n2, np.int64)])
    out["id"] = np.arange(n1 + n2, dtype=np.int64)
    out["orbit"] = el
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
