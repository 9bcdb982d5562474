"""Generates tests/golden/ic_tools_n40.npz: the reference's own initial-condition
tools run on a small synthetic star.

    python tests/golden/make_ic_golden.py REFERENCE_ROOT

Compiles change_polytropic_scale/main.cpp and two_body_initial_condition/main.cpp
from the reference tree with g++ (as their Makefiles do, plus -fpermissive for
their `fp == false` test that current g++ rejects) into a temporary
directory, writes a 40-particle star in the tools' 49-column input format
(1 Msun in total, cgs), and runs:
  * change_scale.out star.data  -> final.data (49 columns, "%lf")
  * two_body_initial.out star.data, answering 1 input file -> two_body.00_t000
    .data (26 columns, "%e") and .head
Their parameters are fixed in each tool's user_define.hpp; they are parsed from
there and stored beside the outputs.  The tools read at least 18 lines
(their composition loop indexes particles 0..17), hence 40 particles.
"""
import glob
import math
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

N = 40
MSUN, RSUN = 1.989e33, 695700e5


def user_defines(path):
    """`double name = expr;` lines of a user_define.hpp, evaluated in order."""
    env = {"sqrt": math.sqrt}
    for name, expr in re.findall(r"^\s*double\s+(\w+)\s*=\s*([^;]+);", open(path).read(), re.M):
        env[name] = float(eval(expr, {"__builtins__": {}}, env))
    return {k: v for k, v in env.items() if k != "sqrt"}


def star_columns(seed=3):
    """49 input columns: id istar mass pos vel acc uene alph alphu dens ksr np
    vsnd pres emp divv rotv bswt pot abar zbar enuc vsmx udot dnuc cmps[18]."""
    rng = np.random.default_rng(seed)
    c = np.zeros((N, 49))
    c[:, 0] = np.arange(N)
    c[:, 2] = MSUN / N
    c[:, 3:6] = rng.uniform(-0.6, 0.6, size=(N, 3)) * RSUN
    c[:, 6:9] = rng.normal(size=(N, 3)) * 3.0e5
    c[:, 9:12] = rng.normal(size=(N, 3)) * 1.0e3
    c[:, 12] = rng.uniform(1e14, 5e15, size=N)
    c[:, 13] = 1.0
    c[:, 15] = rng.uniform(0.1, 10.0, size=N)
    c[:, 16] = rng.uniform(0.1, 0.4, size=N) * RSUN
    c[:, 17] = 50
    c[:, 31 + 1] = c[:, 31 + 2] = 0.5
    return c


def main(ref_root):
    scale_dir = os.path.join(ref_root, "change_polytropic_scale")
    body_dir = os.path.join(ref_root, "two_body_initial_condition")
    star = star_columns()
    with tempfile.TemporaryDirectory() as tmp:
        data = os.path.join(tmp, "star.data")
        with open(data, "w") as f:
            for row in star:
                f.write(f"{int(row[0])} {int(row[1])} " + " ".join(f"{v:.10e}" for v in row[2:]) + "\n")
        star = np.loadtxt(data, ndmin=2)   # the values exactly as the tools read them
        exe = {}
        for name, d in (("change_scale.out", scale_dir), ("two_body_initial.out", body_dir)):
            exe[name] = os.path.join(tmp, name)
            subprocess.run(["g++", "-O2", "-w", "-fpermissive", "-o", exe[name], os.path.join(d, "main.cpp"), "-lm"], check=True)
        subprocess.run([exe["change_scale.out"], data], cwd=tmp, check=True, capture_output=True)
        subprocess.run([exe["two_body_initial.out"], data], cwd=tmp, check=True, capture_output=True,
                       input=b"1\n")
        scaled = np.loadtxt(glob.glob(os.path.join(tmp, "snap_*", "final.data"))[0], ndmin=2)
        prefix = glob.glob(os.path.join(tmp, "data_*", "two_body.00_t000.data"))[0][:-5]
        two_body = np.loadtxt(prefix + ".data", ndmin=2)
        head = open(prefix + ".head").read()
    sd, bd = user_defines(os.path.join(scale_dir, "user_define.hpp")), user_defines(os.path.join(body_dir, "user_define.hpp"))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ic_tools_n40.npz")
    np.savez_compressed(
        out, star=star, scaled=scaled, two_body=two_body, two_body_head=np.array(head),
        scale_m_mul=sd["m_mul"], scale_r_mul=sd["r_mul"],
        orbit_m1=bd["m1"], orbit_m2=bd["m2"], orbit_G=bd["G"], orbit_r_peri=bd["r_rel_p"],
        orbit_v_inf=bd["v_rel_inf"], orbit_r_sep=bd["r_rel"])
    print(out, scaled.shape, two_body.shape)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit(f"usage: python {os.path.relpath(__file__)} <reference root>")
    main(sys.argv[1])
