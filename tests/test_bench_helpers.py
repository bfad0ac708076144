"""CPU checks of bench.py's roofline arithmetic (no device needed)."""
import json

import pytest

import bench


def test_fp64_issue_rate():
    # 72 FP64 instructions per cell, 16.78 M cells in 2.6 ms against 2 x 152 x 2.07 GHz
    r = bench.fp64_issue("predictor", 256 ** 3, 2.6)
    assert r["peak"] == pytest.approx(629.3, abs=0.1)
    assert r["achieved"] == pytest.approx(72 * 256 ** 3 / 2.6e-3 / 1e9, rel=1e-3)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"], rel=1e-3)
    assert bench.fp64_issue("no such kernel", 1, 1.0) is None
    assert bench.fp64_issue("predictor", 1, 0.0) is None


def test_measured_peaks_file_and_fallback(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.measured_peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6660.6}))
    assert bench.measured_peaks() == (6660.6, "measured")


def test_replica_throughput_is_whole_job():
    # N replicas of the same grid finishing within the slowest rank's time
    assert bench.replica_throughput(4, 1000, 10, 2.0) == pytest.approx(4 * 1000 * 10 / 2e-3 / 1e6)
