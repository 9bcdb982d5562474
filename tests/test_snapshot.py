"""The reference's particle file formats: checkpoints (bit-exact), snapshots
and initial conditions.  Host-only code of the engine library, no GPU."""
import numpy as np

from research_codes_gb300 import snapshot as S


def _fields(n, seed=0):
    rng = np.random.default_rng(seed)
    f = {"id": rng.permutation(n).astype(np.int64) * 7 + 3, "istar": rng.integers(0, 2, n).astype(np.int64),
         "mass": rng.random(n) * 3.0, "np": rng.integers(20, 120, n).astype(np.float64)}
    for k in ("pos", "vel", "acc", "acch", "accg1", "accg2"):
        f[k] = rng.normal(size=(n, 3)) * 10.0 ** rng.uniform(-3, 5, size=(n, 3))
    for k in ("uene", "udot", "alph", "adot", "alphu", "adotu", "dens", "pres", "vsnd", "divv", "rotv", "bswt",
              "ksr", "grdh", "vsmx", "pot"):
        f[k] = rng.normal(size=n) * 10.0 ** rng.uniform(-8, 8, size=n)
    return f


def test_hexa_rows_bit_exact(tmp_path):
    f = _fields(257)
    # awkward values: signed zeros, subnormal, huge, non-finite
    f["uene"][:6] = [0.0, -0.0, 5e-324, 1.7976931348623157e308, np.inf, np.nan]
    run = S.default_run(257, time=1234.5, dt=0.0078125, ksr_max=321.25, eps_u=1e-9)
    text = S.hexa_header_text(run) + S.hexa_rows_text(f)
    path = str(tmp_path / "t0000_p000000.hexa")
    open(path, "wb").write(text)
    r2, f2 = S.read_hexa(path)
    for k in ("pos", "vel", "acc", "acch", "accg1", "accg2", "mass", "ksr", "dens", "pot"):
        assert np.array_equal(f2[k].view(np.uint64), np.asarray(f[k], np.float64).view(np.uint64)), k
    assert np.array_equal(f2["uene"].view(np.uint64), f["uene"].view(np.uint64))
    assert np.array_equal(f2["id"], f["id"]) and np.array_equal(f2["istar"], f["istar"])
    for k in ("Time", "Timestep", "KernelSupportRadiusMaximum", "EpsilonOfInternalEnergy", "AlphaMinimum"):
        assert r2[k] == run[k], k
    assert r2["NumberOfSPH"] == 257


def test_hexa_layout_matches_reference_writer():
    """One particle row and the header, as the reference's fprintf calls lay
    them out (hdr_hgas.hpp:286-316, 890-926): "%6lld %2lld %llx" then " %llx"
    per value; header lines in the writer's grouping."""
    f = _fields(1, seed=3)
    f["id"][:] = 42
    f["istar"][:] = 1
    row = S.hexa_rows_text(f).decode()
    tok = row.split()
    assert row.startswith("    42  1 ") and row.endswith("\n")
    assert len(tok) == 2 + len(S.HEXA_COLUMNS) == 2 + 1 + 18 + 22 + 13 + 3
    assert int(tok[2], 16) == int(np.float64(f["mass"][0]).view(np.uint64))
    assert int(tok[3], 16) == int(np.float64(f["pos"][0, 0]).view(np.uint64))
    head = S.hexa_header_text(S.default_run(1, time=2.0, dt=0.5)).decode().split("\n")
    assert head[0].split() == ["4000000000000000", "4000000000000000", "3fe0000000000000",
                               format(int(np.float64(10.0).view(np.uint64)), "x"),
                               format(int(np.float64(10.0).view(np.uint64)), "x"), "0"]
    assert [len(line.split()) for line in head[:10]] == [6, 2, 4, 4, 4, 3, 2, 1, 4, 2]
    assert head[9].startswith(" ")


def test_snapshot_columns_and_format(tmp_path):
    f = _fields(31, seed=5)
    text = S.snapshot_text(f).decode().splitlines()
    assert len(text) == 31
    for i, line in enumerate(text):
        tok = line.split()
        assert len(tok) == 49
        # same printf formats as Python's %-formatting of the cgs values
        assert line[:6] == "%6d" % f["id"][i] and line[6:9] == " %2d" % f["istar"][i]
        assert tok[2] == "%+e" % (f["mass"][i] * S.U_MASS)
        assert tok[3:6] == ["%+e" % (v * S.U_LENGTH) for v in f["pos"][i]]
        assert tok[9:12] == ["%+e" % (v * S.U_ACCELERATION) for v in f["acc"][i]]
        assert tok[17] == "%d" % int(f["np"][i])
        assert tok[33] == "+5.000e-01" and tok[31] == "+0.000e+00"   # composition, " %+.3e"
    path = str(tmp_path / "sph_t0000.dat")
    open(path, "w").write("\n".join(text) + "\n")
    r = S.read_snapshot(path)
    assert np.allclose(r["pos"], f["pos"], rtol=1e-6, atol=0)
    assert np.allclose(r["dens"], f["dens"], rtol=1e-6, atol=0)


def test_initial_conditions_roundtrip(tmp_path):
    rng = np.random.default_rng(2)
    n = 50
    d = {"id": np.arange(n), "istar": np.zeros(n, np.int64), "mass": np.full(n, 1e6 / n),
         "pos": rng.normal(size=(n, 3)) * 700.0, "vel": rng.normal(size=(n, 3)),
         "uene": rng.random(n) * 1e5, "alph": np.ones(n), "alphu": np.zeros(n), "ksr": rng.random(n) * 80.0}
    prefix = str(tmp_path / "two_body.00_t000")
    S.write_data(prefix + ".data", d)
    h = {"Time": 0.0, "TimeEnd": 1e6, "TimestepAscii": 1e4, "TimestepHexa": 1e4, "FlagDamping": 0,
         "FlagNuclear": 0, "AlphaMaximum": 2.0, "AlphaMinimum": 0.1, "AlphuMaximum": 0.0, "AlphuMinimum": 0.0,
         "CoefficientOfTimestep": 0.1, "NumberOfParticle": n}
    S.write_head(prefix + ".head", h)
    h2, d2 = S.read_ic(prefix)
    assert h2 == h
    for k in ("mass", "pos", "vel", "uene", "ksr"):
        assert np.allclose(d2[k], d[k], rtol=1e-6, atol=0), k
    assert np.array_equal(d2["cmps"], S.default_cmps(n))
    assert S.snapshot_path("snap", 7) == "snap/sph_t0007.dat"
    assert S.hexa_path("snap", 3) == "snap/t0003_p000000.hexa"
