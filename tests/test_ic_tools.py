"""CPU tests of the initial-condition tools beyond the polytrope: rescaling a
relaxed star and placing two stars on an unbound Kepler orbit, pinned by the
reference's own change_polytropic_scale and two_body_initial_condition tools
(tests/golden/ic_tools_n40.npz, made by tests/golden/make_ic_golden.py)."""
import math
import os

import numpy as np
import pytest

from research_codes_gb300 import ic, snapshot as S, units

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ic_tools_n40.npz")


def _star_cgs(cols):
    """The tools' 49 input columns as an ic-style dict (cgs)."""
    return {"mass": cols[:, 2].copy(), "pos": cols[:, 3:6].copy(), "vel": cols[:, 6:9].copy(),
            "uene": cols[:, 12].copy(), "ksr": cols[:, 16].copy(), "dens": cols[:, 15].copy(),
            "alph": cols[:, 13].copy(), "alphu": cols[:, 14].copy()}


def test_rescale_matches_the_reference_tool():
    z = np.load(GOLDEN)
    s = ic.rescale(_star_cgs(z["star"]), float(z["scale_m_mul"]), float(z["scale_r_mul"]))
    ref = z["scaled"]
    # the tool prints "%lf": six decimals of cgs values
    for key, cols in (("mass", 2), ("pos", slice(3, 6)), ("vel", slice(6, 9)), ("uene", 12), ("ksr", 16)):
        assert np.allclose(s[key], ref[:, cols], rtol=1e-12, atol=1e-6), key
    # everything else on the line passes through (the tool leaves density as read)
    assert np.array_equal(ref[:, 0], z["star"][:, 0])
    assert np.allclose(ref[:, 13:16], z["star"][:, 13:16], rtol=1e-9, atol=1e-6)


def test_unbound_orbit_matches_the_reference_tool(tmp_path):
    z = np.load(GOLDEN)
    star = _star_cgs(z["star"])
    G, v_inf = float(z["orbit_G"]), float(z["orbit_v_inf"])
    r_peri, r_sep = float(z["orbit_r_peri"]), float(z["orbit_r_sep"])
    # the tool takes its masses from its parameters; the star file sums to them
    assert abs(star["mass"].sum() - float(z["orbit_m1"])) < 1e-9 * float(z["orbit_m1"])
    s = ic.two_stars_on_orbit(star, star, r_peri, v_inf, r_sep, G=G)
    ref = z["two_body"]
    n = len(star["mass"])
    assert ref.shape == (2 * n, 26)
    # "%e" keeps seven significant digits
    for key, cols in (("pos", slice(3, 6)), ("vel", slice(6, 9))):
        scale = np.abs(ref[:, cols]).max()
        assert np.allclose(s[key], ref[:, cols], rtol=1e-6, atol=1e-6 * scale), key
    assert np.array_equal(s["id"], ref[:, 0].astype(np.int64))
    # written through the IC writer (code units -> cgs, "%e"), the whole line
    # equals the tool's, but for istar: the tool copies the input's star index
    # (0 for both copies of one file), this placement numbers the stars 0 / 1
    d = {"id": s["id"], "istar": s["istar"], "mass": s["mass"] / S.U_MASS, "pos": s["pos"] / S.U_LENGTH,
         "vel": s["vel"] / S.U_VELOCITY, "uene": s["uene"] / S.U_ENERGY, "ksr": s["ksr"] / S.U_LENGTH,
         "alph": np.concatenate([star["alph"]] * 2), "alphu": np.concatenate([star["alphu"]] * 2)}
    path = str(tmp_path / "two_body.00_t000.data")
    S.write_data(path, d)
    ours = np.loadtxt(path)
    keep = [c for c in range(26) if c != 1]
    assert np.allclose(ours[:, keep], ref[:, keep], rtol=2e-6, atol=1e-6 * np.abs(ref[:, 3:9]).max())
    assert np.array_equal(ours[:, 1], np.repeat([0, 1], n))
    # the tool's header: t = 0 .. 1e6 s, output every 1e4 s, 2N particles
    hp = str(tmp_path / "two_body.00_t000.head")
    open(hp, "w").write(str(z["two_body_head"]))
    h = S.read_head(hp)
    assert h["NumberOfParticle"] == 2 * n and h["Time"] == 0.0
    assert abs(h["TimeEnd"] - 1e6 * S.U_TIME_INV) < 1e-9 and h["CoefficientOfTimestep"] == 0.1
    S.write_head(hp, h)
    assert S.read_head(hp) == h


@pytest.mark.parametrize("v_inf_kms, peri, sep", [(20.0, 1.5, 10.0), (300.0, 0.3, 4.0), (0.0, 1.0, 6.0),
                                                  (5.0, 2.0, 2.0)])
def test_unbound_orbit_elements(v_inf_kms, peri, sep):
    """Energy, angular momentum and pericentre of the placed pair (code
    units), including the parabola (v_inf = 0) and a start at pericentre."""
    m1, m2 = 1e6, 3e5                     # 1 and 0.3 Msun in code units
    R = 1e3                               # 1 Rsun in code units
    v_inf = v_inf_kms * 1e5 / S.U_VELOCITY
    x1, x2, v1, v2, el = ic.unbound_orbit(m1, m2, peri * R, v_inf, sep * R)
    mu = units.G * (m1 + m2)
    r, v = x1 - x2, v1 - v2
    assert np.allclose(m1 * x1 + m2 * x2, 0.0, atol=1e-12 * sep * R * m1)
    assert np.allclose(m1 * v1 + m2 * v2, 0.0, atol=1e-12 * np.linalg.norm(v) * m1)
    assert abs(np.linalg.norm(r) - sep * R) < 1e-12 * sep * R
    energy = 0.5 * v @ v - mu / np.linalg.norm(r)
    assert abs(energy - 0.5 * v_inf ** 2) < 1e-12 * mu / (peri * R)
    h = np.cross(r, v)
    assert abs(h[2] - el["h"]) < 1e-12 * el["h"] and h[0] == 0.0 and h[1] == 0.0
    assert abs(el["p"] / (1.0 + el["e"]) - peri * R) < 1e-12 * peri * R
    if v_inf > 0:
        assert abs(el["b"] * v_inf - el["h"]) < 1e-12 * el["h"] and el["e"] > 1.0
    else:
        assert el["e"] == 1.0 and math.isinf(el["b"])
    assert (r @ v <= 1e-9 * np.linalg.norm(r) * np.linalg.norm(v))   # approaching (or at pericentre)
    if sep == peri:
        assert abs(el["f"]) < 1e-6


def test_unbound_orbit_rejects_a_start_inside_pericentre():
    with pytest.raises(ValueError):
        ic.unbound_orbit(1e6, 1e6, 2e3, 0.1, 1e3)
    with pytest.raises(ValueError):
        ic.unbound_orbit(1e6, 1e6, 2e3, -0.1, 4e3)


def test_rescaled_polytrope_stays_on_its_adiabat():
    s = ic.polytrope(2000, 1.0, 1.0, 1.5, seed=4)
    t = ic.rescale(s, 10.0, 4.0)
    assert abs(t["M"] - 10.0 * s["M"]) < 1e-12 * t["M"] and abs(t["R"] - 4.0 * s["R"]) < 1e-12 * t["R"]
    assert abs(t["mass"].sum() - t["M"]) < 1e-12 * t["M"]
    # u = n_eos K rho^(1/n) holds with the scaled K, density and energy
    assert np.allclose(t["uene"], units.EOS_N * t["K"] * t["dens"] ** (1.0 / 1.5), rtol=1e-12)
    # the same polytrope built directly at (10 Msun, 4 Rsun) has the same K
    d = ic.polytrope(2000, 10.0, 4.0, 1.5, seed=4)
    assert abs(d["K"] - t["K"]) < 1e-9 * d["K"]
    assert np.allclose(d["pos"], t["pos"], rtol=1e-9, atol=1e-9 * t["R"])
    assert np.allclose(d["uene"], t["uene"], rtol=1e-9)


# ---- the polytropic-star generator (polytropic_initial_condition/) -------------

def test_polytrope_pinned_to_the_reference_generator():
    """ic.polytrope against the reference's own generator, run as shipped
    (tests/golden/make_polytrope_golden.py; 1 Msun, 1 Rsun, n = 1.5):

    * the Lane-Emden table (lane_emden.hpp:14-53, RK4 from r0 = 1e-4, dr =
      1e-3): the tool stores theta after each step against the step's start
      radius, so its row k holds our theta at row k + 1;
    * the polytropic constant and central density (main.cpp:205-213), which
      the tool takes at its last table row instead of the exact first zero;
    * the density theta^n of a particle at the tool's table index;
    * the radial map from enclosed-mass fraction to Lane-Emden radius: given
      the tool's own mass profile, our interpolation lands on the tool's
      binary-search radius to within one table step.
    Deliberate differences (documented in ic.py): the tool integrates theta
    rather than rho = theta^n for the mass profile (main.cpp:107-110) and
    writes u = n P (main.cpp:225); the lattice here has a seeded phase and
    rotation."""
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "polytrope_tool_n15.npz")))
    n = float(g["n_index"])
    xi, th, dth, a, rho_c, K = ic.polytrope_scalings(n, float(g["mass"]), float(g["radius"]), float(g["G"]))
    dr, r0 = 1e-3, 1e-4
    rows = np.round((g["le_r"] - r0) / dr).astype(int)
    assert np.abs(xi[rows] - g["le_r"]).max() < 1e-6
    assert np.abs(th[rows + 1] - g["le_theta"]).max() < 1e-6
    assert np.abs(dth[rows + 1] - g["le_dtheta"]).max() < 1e-6
    assert int(g["le_rows"]) == len(xi) - 2        # the tool stops one row before the zero
    # K and rho_c: the tool's ones from its last row, ours from the exact zero
    r_last, th_last, v_last = g["le_last"]
    rho_ave = 3.0 * float(g["mass"]) / (4.0 * np.pi * float(g["radius"]) ** 3)
    rho_c_tool = -rho_ave / (3.0 * v_last / r_last)
    G, R = float(g["G"]), float(g["radius"])
    k_tool = 4 * np.pi * G * R * R * rho_c_tool ** ((n - 1) / n) / ((n + 1) * r_last * r_last)
    assert k_tool == pytest.approx(float(g["k_cgs"]), rel=1e-6)     # printed with 7 digits
    assert K == pytest.approx(k_tool, rel=2e-3)
    assert rho_c == pytest.approx(rho_c_tool, rel=2e-3)
    # density at the tool's table index: rho_c theta(index + 1)^n
    lane = g["sp_lane"].astype(int)
    dens = rho_c_tool * th[lane + 1] ** n
    assert np.allclose(dens, g["real_dens"], rtol=1e-5, atol=6e-7)   # printed with 6 decimals
    # P = K rho^(1 + 1/n) and c^2 = (1 + 1/n) P / rho; the tool's u = n P
    pres = k_tool * dens ** (1 + 1 / n)
    big = g["real_pres"] > 1e7
    assert np.allclose(g["real_pres"][big], pres[big], rtol=1e-5)
    assert np.allclose(g["real_vsnd"][big], np.sqrt((1 + 1 / n) * pres / dens)[big], rtol=1e-5)
    assert np.allclose(g["real_uene"][big], n * pres[big], rtol=1e-5)
    # radial map with the tool's mass profile (cumulative 4/3 pi dr^3 theta)
    rt, tt = xi[:-1][: int(g["le_rows"])], th[1:][: int(g["le_rows"])]
    m = np.empty(len(rt))
    m[0] = rt[0] ** 3 * tt[0]
    m[1:] = m[0] + np.cumsum((rt[1:] ** 3 - rt[:-1] ** 3) * tt[1:])
    m /= m[-1]
    r_map = np.interp(g["sp_mfrac"], m, rt)
    assert np.abs(r_map - g["sp_r_pori"]).max() < 2.5 * dr
