"""CPU checks of the bench line's host-side parts: profile-derived figures,
the clock sampler's parsing and the CPU-baseline rate mix (no GPU)."""
import json

import bench


def test_tree_lists_rate_from_the_committed_capture(tmp_path):
    r = bench.tree_lists_rate()
    assert r is not None
    assert r["dram_bytes"] > 0 and r["ncu_ms"] > 0
    assert abs(r["achieved_gbs"] - r["dram_bytes"] / (r["ncu_ms"] * 1e-3) / 1e9) < 1e-9 * r["achieved_gbs"]
    assert 0.0 < r["frac"] < 1.0   # latency-bound kernels, far below the copy rate
    assert set(r["groups"]) == {"tree", "lists"}
    # without a measured peak the fallback copy rate is used and named
    r2 = bench.tree_lists_rate(peaks_path=str(tmp_path / "absent.json"))
    assert r2["peak_gbs"] == 6800.0 and "fallback" in r2["peak_source"]
    peaks = tmp_path / "peaks.json"
    peaks.write_text(json.dumps({"hbm_gbs": 5000.0}))
    r3 = bench.tree_lists_rate(peaks_path=str(peaks))
    assert r3["peak_gbs"] == 5000.0 and abs(r3["frac"] - r3["achieved_gbs"] / 5000.0) < 1e-12


def test_tree_lists_rate_without_a_capture(tmp_path):
    p = tmp_path / "traffic.json"
    p.write_text(json.dumps({"gravity": {"bytes_per_launch": 1}}))
    assert bench.tree_lists_rate(traffic_path=str(p)) is None
    assert bench.tree_lists_rate(traffic_path=str(tmp_path / "missing.json")) is None


def test_pair_kernel_traffic_entries():
    tr = json.load(open(bench.PROFILE_TRAFFIC))
    for k in ("density", "hydro_signal", "hydro_df", "gravity"):
        assert tr[k]["bytes_per_launch"] == round(tr[k]["read"] + tr[k]["write"])
        assert tr[k]["ncu_ms"] > 0


class _FakeSmi:
    """Stands in for `nvidia-smi --query-gpu=... -lms 200`: yields fixed lines."""
    lines = []

    def __init__(self, *a, **kw):
        import io
        self.stdout = io.StringIO("".join(self.lines))

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def test_clock_sampler_parses_samples_and_reasons(monkeypatch):
    _FakeSmi.lines = [
        "1965, 2070, 900.10, Not Active, Not Active, Not Active, Not Active\n",
        "1980, 2070, 1201.5, Not Active, Not Active, Not Active, Active\n",
        "[N/A], [N/A], [N/A], Not Active, Not Active, Not Active, Not Active\n",
        "2010, 2070, 1100.0, Not Active, Not Active, Not Active, Not Active\n",
        "garbage\n",
    ]
    monkeypatch.setattr(bench.subprocess, "Popen", _FakeSmi)
    c = bench.ClockSampler()
    c.start()
    c.thread.join(timeout=5)
    r = c.stop()
    assert r["samples"] == 4                 # the malformed line is dropped
    assert r["sm_mhz"] == 1980.0 and r["sm_max_mhz"] == 2070.0   # median of the numeric samples
    assert r["reasons"] == ["sw_power_cap"]


def test_clock_sampler_without_nvidia_smi(monkeypatch):
    def missing(*a, **kw):
        raise FileNotFoundError("nvidia-smi")
    monkeypatch.setattr(bench.subprocess, "Popen", missing)
    c = bench.ClockSampler()
    c.start()
    assert c.stop() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}


def test_combined_rate_is_the_pair_weighted_harmonic_mean():
    rates = {"density": (1e9, 1.0), "hydro": (4e9, 2.0)}     # 1e9 and 2e9 pairs/s
    assert abs(bench.combined_rate(rates, {"density": 1, "hydro": 1}) - 2 / (1 / 1e9 + 1 / 2e9)) < 1e-3
    assert abs(bench.combined_rate(rates, {"density": 3, "hydro": 0}) - 1e9) < 1e-3


def _run_reference_arm(rank, tmp_path):
    import os
    import subprocess
    import sys
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2" if rank else "1", OMP_NUM_THREADS="2")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    return subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--config", "c0",
                           "--scale", "0.2", "--steps", "1", "--warmup", "0"],
                          cwd=str(tmp_path), env=env, capture_output=True, text=True, timeout=300)


def test_reference_arm_prints_one_contract_line(tmp_path):
    p = _run_reference_arm(0, tmp_path)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    r = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in r, k
    assert r["impl"] == "reference" and r["value"] > 0 and r["warmup"] >= 3
    assert r["unit"] == "s/step" and r["higher_is_better"] is False
    assert r["cpu_baseline"]["kind"] == "port" and r["cpu_baseline"]["value"] == r["value"]
    assert r["e2e"] == {"value": r["value"], "unit": r["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert r["config"]["workload"].startswith("c0: single n=1.5 polytrope")


def test_reference_arm_other_ranks_exit_quietly(tmp_path):
    p = _run_reference_arm(1, tmp_path)
    assert p.returncode == 0 and p.stdout.strip() == ""
