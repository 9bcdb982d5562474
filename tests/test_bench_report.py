"""CPU checks of the bench line's profile-derived figures (no GPU)."""
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
    for k in ("density", "hydro", "gravity"):
        assert tr[k]["bytes_per_launch"] == round(tr[k]["read"] + tr[k]["write"])
        assert tr[k]["ncu_ms"] > 0
