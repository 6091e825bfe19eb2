"""The bench's roofline arithmetic on the CPU: algorithmic bytes per launch, achieved
bandwidth from event time, the fraction of the measured peak and the DRAM traffic scaled
from the committed capture."""

import json
import os
import sys

REPO = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
sys.path.insert(0, REPO)
import bench  # noqa: E402


def test_per_launch_bytes():
    b = bench.per_launch_bytes(neq=10, nnz=100, tri=3, nodes=7, w=4, wx=4)
    assert b["spmv"] == 100 * 8 + 4 * 11 + 2 * 10 * 4
    assert b["trsv"] == (100 * 8 + 4 * 11 + 3 * 10 * 4) / 2
    assert b["factor"] == 2 * 100 * 4 + 4 * 100 + 4 * 11
    assert b["assemble"] == 100 * 4 + 8 * 10 + 120 * 7 + 24 * 3 + 900 * 3


def test_class_rooflines_and_trsv_roofline(tmp_path, monkeypatch):
    peaks = tmp_path / "peaks.json"
    peaks.write_text(json.dumps({"hbm_gbs": 1000.0}))
    monkeypatch.setattr(bench, "PEAKS_FILE", str(peaks))
    traffic = tmp_path / "traffic.json"
    traffic.write_text(json.dumps({"neq": 5, "bytes_per_launch": 2.0e6}))
    monkeypatch.setattr(bench, "TRAFFIC_FILE", str(traffic))
    neq, nnz = 1_000_000, 30_000_000
    per = bench.per_launch_bytes(neq, nnz, 0, 0, 4, 4)
    # 100 launches in 200 ms: 2 ms each
    prof = {"trsv": (100, 200.0), "spmv": (10, 5.0), "factor": (0, 0.0), "assemble": (1, 10.0)}
    cls = bench.class_rooflines(prof, neq, nnz, 0, 0, 4, 4)
    assert cls["peak_gbs"] == 1000.0 and cls["peak_kind"] == "measured"
    t = cls["classes"]["trsv"]
    assert t["avg_launch_ms"] == 2.0
    assert abs(t["achieved_gbs"] - per["trsv"] / 2e-3 / 1e9) < 0.01
    assert abs(t["frac"] - t["achieved_gbs"] / 1000.0) < 1e-5
    assert "factor" not in cls["classes"]          # no launches, no entry
    r = bench.trsv_roofline(prof, neq, nnz, 0, 0, dev_ms_total=400.0)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["peak"] == 1000.0
    assert abs(r["achieved"] - per["trsv"] / 2e-3 / 1e9) < 0.01
    assert r["traffic"] == 2.0e6 * neq / 5            # scaled by the equation count
    assert r["share_of_step_device_time"] == 0.5


def test_peak_falls_back_without_the_measured_file(monkeypatch, tmp_path):
    monkeypatch.setattr(bench, "PEAKS_FILE", str(tmp_path / "absent.json"))
    peak, kind = bench.hbm_peak()
    assert kind == "fallback" and peak == bench.FALLBACK_HBM_GBS


def test_committed_traffic_file_is_a_capture_of_the_window():
    with open(bench.TRAFFIC_FILE) as f:
        tr = json.load(f)
    assert tr["neq"] == 476424 and tr["bytes_per_launch"] > 0 and "ncu" in tr["source"]
