"""The reference's particle files, read and written in its own formats.

* Initial conditions: ``<name>.head`` (run parameters, RunParameter::readAscii,
  hdr_hgas.hpp:775-800) and ``<name>.data`` (one line per particle,
  HelmholtzGas::readAscii, hdr_hgas.hpp:115-134), in cgs units.
* Snapshots ``snap/sph_tNNNN.dat``: 49 columns per particle in cgs units
  (HelmholtzGas::writeAscii, hdr_hgas.hpp:136-180), written every
  TimestepAscii (outputData, hdr_hgas.hpp:1026-1050).
* Checkpoints ``snap/tNNNN_pNNNNNN.hexa``: the run header
  (RunParameter::writeHexa, hdr_hgas.hpp:890-926) and every FP64 value of the
  particle state as the hexadecimal image of its bits
  (HelmholtzGas::writeHexa, hdr_hgas.hpp:286-316), so that a restart
  continues bit for bit (restartSimulation, hdr_hgas.hpp:1383-1412, reads it
  back without a new force evaluation).

The per-particle text is produced and parsed by the engine library
(``sph_format_hexa_rows``, ``sph_parse_hexa_rows``, ``sph_format_ascii_rows``).
Values the ideal-gas path does not compute (temperature, composition,
nuclear energy, ...) are written as the reference's initial values for them:
zero, composition as read (0.5 / 0.5 carbon-oxygen from the IC tools).
"""
import ctypes
import os

import numpy as np

from . import _lib, units

N_CMPS = 13   # NuclearReaction::NumberOfNucleon, hdr_heos.hpp:115

# Unit conversions exactly as the reference forms them (hdr_heos.hpp:67-91).
U_LENGTH = units.SOLAR_RADIUS * 1.0e-3
U_MASS = units.SOLAR_MASS * 1.0e-6
U_TIME = 1.0
U_VELOCITY = U_LENGTH / U_TIME
U_DENSITY = U_MASS / (U_LENGTH * U_LENGTH * U_LENGTH)
U_ENERGY = U_VELOCITY * U_VELOCITY
U_PRESSURE = U_MASS * U_LENGTH / (U_TIME * U_TIME * U_LENGTH * U_LENGTH)
U_ACCELERATION = U_VELOCITY / U_TIME
U_LENGTH_INV, U_MASS_INV, U_TIME_INV = 1.0 / U_LENGTH, 1.0 / U_MASS, 1.0 / U_TIME
U_VELOCITY_INV, U_ENERGY_INV = 1.0 / U_VELOCITY, 1.0 / U_ENERGY


def _declare():
    lib = _lib.load()
    P, I64, I32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
    lib.sph_format_hexa_rows.restype = I64
    lib.sph_format_hexa_rows.argtypes = [I64, P, P, I32, P, P, I64]
    lib.sph_parse_hexa_rows.restype = I64
    lib.sph_parse_hexa_rows.argtypes = [P, I64, I64, I32, P, P, P]
    lib.sph_format_ascii_rows.restype = I64
    lib.sph_format_ascii_rows.argtypes = [I64, P, P, I32, P, ctypes.c_char_p, P, I64]
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _text(fn, *args):
    """Runs a sph_format_* function twice: size, then fill."""
    need = fn(*args, None, 0)
    if need < 0:
        raise ValueError(f"bad arguments (status {-need})")
    buf = ctypes.create_string_buffer(int(need) + 1)
    got = fn(*args, buf, need + 1)
    if got != need:
        raise RuntimeError("text encoder returned an inconsistent size")
    return buf.raw[:need]


# ----------------------------------------------------------------- initial conditions
HEAD_KEYS = ("Time", "TimeEnd", "TimestepAscii", "TimestepHexa", "FlagDamping", "FlagNuclear",
             "AlphaMaximum", "AlphaMinimum", "AlphuMaximum", "AlphuMinimum", "CoefficientOfTimestep",
             "NumberOfParticle")


def read_head(path):
    """RunParameter::readAscii: times in s, converted to code units."""
    tok = open(path).read().split()
    if len(tok) < len(HEAD_KEYS):
        raise ValueError(f"{path}: {len(tok)} values, {len(HEAD_KEYS)} expected")
    h = {}
    for k, v in zip(HEAD_KEYS, tok):
        h[k] = int(v) if k in ("FlagDamping", "FlagNuclear", "NumberOfParticle") else float(v)
    for k in ("Time", "TimeEnd", "TimestepAscii", "TimestepHexa"):
        h[k] *= U_TIME_INV
    return h


def write_head(path, h):
    """The header the IC tools write (two_body_initial_condition/main.cpp:193-198)."""
    with open(path, "w") as f:
        f.write(f"{h['Time'] * U_TIME:+e} {h['TimeEnd'] * U_TIME:+e} {h['TimestepAscii'] * U_TIME:e} "
                f"{h['TimestepHexa'] * U_TIME:e}\n")
        f.write(f"{int(h['FlagDamping'])} {int(h['FlagNuclear'])}\n")
        f.write(f"{h['AlphaMaximum']:+e} {h['AlphaMinimum']:+e}\n")
        f.write(f"{h['AlphuMaximum']:+e} {h['AlphuMinimum']:+e}\n")
        f.write(f"{h['CoefficientOfTimestep']:+e}\n")
        f.write(f"{int(h['NumberOfParticle'])}\n")


def read_data(path):
    """HelmholtzGas::readAscii for every line: id istar mass pos vel uene alph
    alphu ksr, then the composition; cgs -> code units by the reference's
    multiplications with the inverse units."""
    raw = np.loadtxt(path, dtype=np.float64, ndmin=2)
    if raw.shape[1] < 13:
        raise ValueError(f"{path}: {raw.shape[1]} columns, at least 13 expected")
    d = {"id": raw[:, 0].astype(np.int64), "istar": raw[:, 1].astype(np.int64),
         "mass": raw[:, 2] * U_MASS_INV, "pos": raw[:, 3:6] * U_LENGTH_INV, "vel": raw[:, 6:9] * U_VELOCITY_INV,
         "uene": raw[:, 9] * U_ENERGY_INV, "alph": raw[:, 10].copy(), "alphu": raw[:, 11].copy(),
         "ksr": raw[:, 12] * U_LENGTH_INV}
    cm = np.zeros((len(raw), N_CMPS))
    k = min(N_CMPS, raw.shape[1] - 13)
    cm[:, :k] = raw[:, 13:13 + k]
    d["cmps"] = cm
    return d


def write_data(path, d):
    """Initial-condition lines as the IC tools print them (cgs, "%e")."""
    n = len(d["mass"])
    cm = d.get("cmps", default_cmps(n))
    with open(path, "w") as f:
        for i in range(n):
            row = [d["mass"][i] * U_MASS, *(d["pos"][i] * U_LENGTH), *(d["vel"][i] * U_VELOCITY),
                   d["uene"][i] * U_ENERGY, d["alph"][i], d["alphu"][i], d["ksr"][i] * U_LENGTH]
            f.write(f"{int(d['id'][i])} {int(d['istar'][i])} " + " ".join(f"{v:e}" for v in row)
                    + "".join(f" {v:e}" for v in cm[i]) + "\n")


def default_cmps(n):
    """Composition of the IC tools: 0.5 carbon, 0.5 oxygen (make_and_output_data.hpp:17-19)."""
    c = np.zeros((n, N_CMPS))
    c[:, 1] = c[:, 2] = 0.5
    return c


def read_ic(prefix):
    """(run parameters, particles) of ``prefix.head`` / ``prefix.data``."""
    return read_head(prefix + ".head"), read_data(prefix + ".data")


# ----------------------------------------------------------------- snapshots
# HelmholtzGas::writeAscii columns after id, istar (3..49), with their scale
# to cgs and print kind; columns the ideal-gas path does not compute are 0.
ASCII_COLUMNS = (
    [("mass", U_MASS, "e")] + [(f"pos{k}", U_LENGTH, "e") for k in range(3)]
    + [(f"vel{k}", U_VELOCITY, "e") for k in range(3)] + [(f"acc{k}", U_ACCELERATION, "e") for k in range(3)]
    + [("uene", U_ENERGY, "e"), ("alph", 1.0, "e"), ("alphu", 1.0, "e"), ("dens", U_DENSITY, "e"),
       ("ksr", U_LENGTH, "e"), ("np", 1.0, "d"), ("vsnd", U_VELOCITY, "e"), ("pres", U_PRESSURE, "e"),
       ("temp", 1.0, "e"), ("divv", U_TIME_INV, "e"), ("rotv", U_TIME_INV, "e"), ("bswt", 1.0, "e"),
       ("pot", U_ENERGY, "e"), ("abar", 1.0, "e"), ("zbar", 1.0, "e"), ("enuc", U_ENERGY, "e"),
       ("vsmx", U_VELOCITY, "e"), ("udot", U_ENERGY * U_TIME_INV, "e"), ("dnuc", U_ENERGY, "e")]
    + [(f"cmps{k}", 1.0, "c") for k in range(N_CMPS)]
    + [("pot3", U_ENERGY, "e"), ("tempmax0", 1.0, "e"), ("tempmax1", U_DENSITY, "e"), ("tempmax2", 1.0, "e"),
       ("entr", U_ENERGY, "e")])
assert len(ASCII_COLUMNS) == 47   # + id, istar = 49


def _column(f, name, n):
    """Array of column `name` from a field dict (code units)."""
    for vec in ("pos", "vel", "acc"):
        if name.startswith(vec) and name[len(vec):].isdigit():
            return np.asarray(f[vec])[:, int(name[len(vec):])]
    if name.startswith("cmps"):
        return np.asarray(f.get("cmps", default_cmps(n)))[:, int(name[4:])]
    if name.startswith("tempmax"):
        return np.asarray(f.get("tempmax", np.zeros((n, 3))))[:, int(name[7:])]
    return np.asarray(f.get(name, np.zeros(n)), dtype=np.float64)


def snapshot_text(f):
    """The bytes of an ``sph_tNNNN.dat`` file for the field dict f (code units)."""
    n = len(f["mass"])
    cols = np.empty((n, len(ASCII_COLUMNS)))
    for k, (name, scale, _) in enumerate(ASCII_COLUMNS):
        cols[:, k] = _column(f, name, n) * scale
    kinds = "".join(c[2] for c in ASCII_COLUMNS).encode()
    ids = np.ascontiguousarray(f["id"], dtype=np.int64)
    ist = np.ascontiguousarray(f.get("istar", np.zeros(n)), dtype=np.int64)
    cols = np.ascontiguousarray(cols)
    lib = _declare()
    return _text(lib.sph_format_ascii_rows, n, _ptr(ids), _ptr(ist), len(ASCII_COLUMNS), _ptr(cols), kinds)


def write_snapshot(path, f):
    with open(path, "wb") as fh:
        fh.write(snapshot_text(f))


def read_snapshot(path):
    """Columns of an ``sph_tNNNN.dat`` file back in code units (decimal text:
    7 significant digits, as written)."""
    raw = np.loadtxt(path, dtype=np.float64, ndmin=2)
    out = {"id": raw[:, 0].astype(np.int64), "istar": raw[:, 1].astype(np.int64)}
    for k, (name, scale, _) in enumerate(ASCII_COLUMNS):
        out[name] = raw[:, 2 + k] / scale
    for vec in ("pos", "vel", "acc"):
        out[vec] = np.stack([out.pop(f"{vec}{k}") for k in range(3)], axis=1)
    out["cmps"] = np.stack([out.pop(f"cmps{k}") for k in range(N_CMPS)], axis=1)
    out["tempmax"] = np.stack([out.pop(f"tempmax{k}") for k in range(3)], axis=1)
    return out


def snapshot_path(directory, number):
    """outputData's name of ASCII snapshot `number` (hdr_hgas.hpp:1036)."""
    return os.path.join(directory, f"sph_t{number:04d}.dat")


# ----------------------------------------------------------------- checkpoints
# HelmholtzGas::writeHexa values after id, istar, in order.
HEXA_COLUMNS = (["mass"] + [f"pos{k}" for k in range(3)] + [f"vel{k}" for k in range(3)]
                + [f"acc{k}" for k in range(3)] + [f"acch{k}" for k in range(3)]
                + [f"accg1{k}" for k in range(3)] + [f"accg2{k}" for k in range(3)]
                + ["uene", "udot", "alph", "adot", "alphu", "adotu", "dens", "pres", "vsnd", "temp",
                   "divv", "rotv", "bswt", "ksr", "grdh", "vsmx", "pot", "enuc", "dnuc", "abar", "zbar", "gcor3"]
                + [f"cmps{k}" for k in range(N_CMPS)] + [f"tempmax{k}" for k in range(3)])
VEC_FIELDS = ("pos", "vel", "acc", "acch", "accg1", "accg2")

# RunParameter::writeHexa header, hdr_hgas.hpp:890-926: (key, 'x' = FP64 as
# hex bits | 'd' = integer) per line.
HEXA_HEADER = ([("Time", "x"), ("TimeEnd", "x"), ("Timestep", "x"), ("TimestepAscii", "x"), ("TimestepHexa", "x"),
                ("NumberOfStep", "d")],
               [("NumberOfAscii", "d"), ("NumberOfHexa", "d")],
               [("AlphaMaximum", "x"), ("AlphaMinimum", "x"), ("AlphuMaximum", "x"), ("AlphuMinimum", "x")],
               [("KernelSupportRadiusMaximum", "x"), ("EpsilonOfInternalEnergy", "x"), ("ReductionTime", "x"),
                ("ReductionTimeInv", "x")],
               [("NumberOfSPH", "d"), ("NumberOfMassless", "d"), ("NumberOfBHNS", "d"),
                ("CoefficientOfTimestep", "x")],
               [("RotationalVelocity0", "x"), ("RotationalVelocity1", "x"), ("RotationalVelocity2", "x")],
               [("NuclearEnergyTotal", "x"), ("AbsorbedEnergyTotal", "x")],
               [("FlagDivideFile", "d")],
               [("FlagDamping", "d"), ("FlagNuclear", "d"), ("FlagBinary", "d"), ("FlagPotential", "d")],
               [("BlackHoleMass", "x"), ("BlackHoleMassInThisUnit", "x")])


def _hex(x):
    return format(int(np.float64(x).view(np.uint64)), "x")


def _unhex(s):
    return float(np.uint64(int(s, 16)).view(np.float64))


def hexa_header_text(run):
    """Header lines; `run` needs every key of HEXA_HEADER and 'domains'
    (one (lo[3], hi[3]) per process)."""
    lines = []
    for k, line in enumerate(HEXA_HEADER):
        vals = [(_hex(run[key]) if t == "x" else str(int(run[key]))) for key, t in line]
        lines.append((" " if k == len(HEXA_HEADER) - 1 else "") + " ".join(vals))
    for lo, hi in run["domains"]:
        lines.append(" ".join(_hex(v) for v in (*lo, *hi)))
    return ("\n".join(lines) + "\n").encode()


def hexa_rows_text(f):
    n = len(f["mass"])
    cols = np.empty((n, len(HEXA_COLUMNS)))
    for k, name in enumerate(HEXA_COLUMNS):
        cols[:, k] = _hexa_column(f, name, n)
    ids = np.ascontiguousarray(f["id"], dtype=np.int64)
    ist = np.ascontiguousarray(f.get("istar", np.zeros(n)), dtype=np.int64)
    lib = _declare()
    return _text(lib.sph_format_hexa_rows, n, _ptr(ids), _ptr(ist), len(HEXA_COLUMNS),
                 _ptr(np.ascontiguousarray(cols)))


def _hexa_column(f, name, n):
    for vec in VEC_FIELDS:
        if name.startswith(vec) and name[len(vec):].isdigit():
            return np.asarray(f.get(vec, np.zeros((n, 3))))[:, int(name[len(vec):])]
    return _column(f, name, n)


def write_hexa(path, run, f):
    with open(path, "wb") as fh:
        fh.write(hexa_header_text(run))
        fh.write(hexa_rows_text(f))


def read_hexa(path, n_proc=1):
    """(run header dict, particle field dict) of a checkpoint; every FP64
    value bit-exact."""
    data = open(path, "rb").read()
    tok = data.split()
    run, pos = {}, 0
    for line in HEXA_HEADER:
        for key, t in line:
            run[key] = _unhex(tok[pos].decode()) if t == "x" else int(tok[pos])
            pos += 1
    run["domains"] = []
    for _ in range(n_proc):
        v = [_unhex(t.decode()) for t in tok[pos:pos + 6]]
        run["domains"].append((v[:3], v[3:]))
        pos += 6
    n = int(run["NumberOfSPH"])
    # byte offset of the first particle row: after the header's tokens
    off = 0
    for _ in range(pos):
        while data[off:off + 1].isspace():
            off += 1
        while off < len(data) and not data[off:off + 1].isspace():
            off += 1
    body = data[off:]
    ids = np.empty(n, np.int64)
    ist = np.empty(n, np.int64)
    cols = np.empty((n, len(HEXA_COLUMNS)))
    lib = _declare()
    got = lib.sph_parse_hexa_rows(body, len(body), n, len(HEXA_COLUMNS), _ptr(ids), _ptr(ist), _ptr(cols))
    if got != n:
        raise ValueError(f"{path}: parsed {got} of {n} particle rows")
    f = {"id": ids, "istar": ist}
    for k, name in enumerate(HEXA_COLUMNS):
        f[name] = cols[:, k]
    for vec in VEC_FIELDS:
        f[vec] = np.stack([f.pop(f"{vec}{k}") for k in range(3)], axis=1)
    f["cmps"] = np.stack([f.pop(f"cmps{k}") for k in range(N_CMPS)], axis=1)
    f["tempmax"] = np.stack([f.pop(f"tempmax{k}") for k in range(3)], axis=1)
    return run, f


def hexa_path(directory, number, rank=0):
    """outputData's name of checkpoint `number` (hdr_hgas.hpp:1057)."""
    return os.path.join(directory, f"t{number:04d}_p{rank:06d}.hexa")


# ----------------------------------------------------------------- system state
# Per-particle results of the last force evaluation that the next step reads
# (time step, predictor) or that a snapshot prints; a restart restores them
# instead of evaluating the forces again, as the reference does.
STATE_FIELDS = ("acc", "acch", "accg1", "accg2", "udot", "adot", "adotu", "dens", "pres", "vsnd", "divv",
                "rotv", "bswt", "grdh", "vsmx", "pot", "eta", "diffu")


def system_fields(ps):
    """Every field of a ParticleSystem in upload order (code units)."""
    f = {k: ps.download(k) for k in ("pos", "vel", "mass", "uene", "alph", "alphu", "ksr", "np") + STATE_FIELDS}
    f["id"] = ps.download("id").astype(np.int64)
    f["istar"] = ps.download("istar").astype(np.int64)
    return f


def default_run(n, time=0.0, dt=10.0, ksr_max=0.0, eps_u=0.0):
    """A checkpoint header for a single-process run of the ideal-gas path."""
    run = {key: 0 for line in HEXA_HEADER for key, _ in line}
    run.update(Time=time, TimeEnd=time, Timestep=dt, TimestepAscii=units.DT_MAX, TimestepHexa=units.DT_MAX,
               AlphaMaximum=units.ALPHA_MAX, AlphaMinimum=units.ALPHA_MIN, AlphuMaximum=units.ALPHU_MAX,
               AlphuMinimum=units.ALPHU_MIN, KernelSupportRadiusMaximum=ksr_max, EpsilonOfInternalEnergy=eps_u,
               NumberOfSPH=n, CoefficientOfTimestep=units.C_DT, domains=[((0.0, 0.0, 0.0), (0.0, 0.0, 0.0))])
    return run


def save_checkpoint(ps, path, run=None):
    """Writes the system's state as a reference checkpoint; the clock (time,
    dt, ksrmax, epsu) goes into the header."""
    f = system_fields(ps)
    time, dt, ksr_max, eps_u = ps.clock()
    r = default_run(ps.n)
    r.update(run or {})
    r.update(Time=time, Timestep=dt, KernelSupportRadiusMaximum=ksr_max, EpsilonOfInternalEnergy=eps_u,
             NumberOfSPH=ps.n)
    write_hexa(path, r, f)
    return r


def load_checkpoint(ps, path):
    """Restores a system from a checkpoint (its size must match): particle
    state, last force results and clock, so that the next step continues the
    run without a new force evaluation.  Returns the header."""
    run, f = read_hexa(path)
    if int(run["NumberOfSPH"]) != ps.n:
        raise ValueError(f"{path}: {run['NumberOfSPH']} particles, system has {ps.n}")
    ps.upload({"id": f["id"], "istar": f["istar"], "mass": f["mass"], "pos": f["pos"], "vel": f["vel"],
               "uene": f["uene"], "ksr": f["ksr"], "alph": f["alph"], "alphu": f["alphu"]}, t0=run["Time"])
    for k in STATE_FIELDS:
        if k in f:
            ps.set_field(k, f[k])
    ps.set_clock(run["Time"], run["Timestep"], run["KernelSupportRadiusMaximum"],
                 run["EpsilonOfInternalEnergy"])
    return run
