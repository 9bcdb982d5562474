"""Generates tests/golden/polytrope_tool_n15.npz: the reference's own
polytropic-star generator run as shipped.

    python tests/golden/make_polytrope_golden.py REFERENCE_ROOT

Compiles polytropic_initial_condition/main.cpp from the reference tree with
g++ (as its Makefile does) into a temporary directory and runs it with its
fixed parameters (user_defined.hpp: 1 Msun, 1 Rsun, n = 1.5, lattice step
0.05).  Stored: every 10th row of its Lane-Emden table (lane_emden.data: r,
theta, theta'), every 16th lattice particle's radius, enclosed-mass
fraction, mapped Lane-Emden radius and table index (sphere.data), the same
particles' density, pressure, sound speed and internal energy in cgs
(real.data), the polytropic constant it prints, and its parameters.
"""
import os
import re
import subprocess
import sys
import tempfile

import numpy as np


def user_defines(path):
    """`double name = expr;` lines, evaluated in order (msun, rsun, G, ...)."""
    env = {}
    for name, expr in re.findall(r"^\s*double\s+(\w+)\s*=\s*([^;]+);", open(path).read(), re.M):
        env[name] = float(eval(expr, {"__builtins__": {}}, env))
    return env


def main(ref_root):
    src = os.path.join(ref_root, "polytropic_initial_condition")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "polytropic_condition.out")
        subprocess.run(["g++", "-O3", "-w", "-o", exe, os.path.join(src, "main.cpp"), "-lm"], check=True)
        p = subprocess.run([exe], cwd=tmp, check=True, capture_output=True, text=True)
        k_cgs = float(re.search(r"k = ([0-9.eE+-]+)", p.stderr).group(1))
        out = os.path.join(tmp, "output_n_1.5")
        le = np.loadtxt(os.path.join(out, "lane_emden.data"), ndmin=2)
        sphere = np.loadtxt(os.path.join(out, "sphere.data"), ndmin=2)
        real = np.loadtxt(os.path.join(out, "real.data"), ndmin=2)
    ud = user_defines(os.path.join(src, "user_defined.hpp"))
    take = np.arange(0, len(sphere), 16)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "polytrope_tool_n15.npz")
    np.savez_compressed(
        path, le_r=le[::10, 1], le_theta=le[::10, 2], le_dtheta=le[::10, 3], le_last=le[-1, 1:4],
        le_rows=np.array(len(le)),
        sp_r=sphere[take, 4], sp_mfrac=sphere[take, 5], sp_r_pori=sphere[take, 9], sp_lane=sphere[take, 11],
        real_r=real[take, 4], real_dens=real[take, 5], real_pres=real[take, 6], real_vsnd=real[take, 7],
        real_uene=real[take, 8], n_particles=np.array(len(sphere)), k_cgs=np.array(k_cgs),
        mass=np.array(ud["MASS"]), radius=np.array(ud["RADIUS"]), G=np.array(ud["G"]),
        n_index=np.array(ud["pori_num"]), lattice_step=np.array(ud["dt"]))
    print("wrote", path, len(sphere), "particles,", len(le), "table rows")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit(f"usage: python {os.path.relpath(__file__)} <reference root>")
    main(sys.argv[1])
