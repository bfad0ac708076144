"""CPU checks of bench.py's roofline arithmetic (no device needed)."""
import json

import pytest

import bench


def test_fp64_issue_rate():
    # 72 FP64 instructions per cell, 16.78 M cells in 2.6 ms against 2 x 152 x 2.07 GHz
    r = bench.fp64_issue(72.0, 256 ** 3, 2.6, sms=152, ghz=2.07)
    assert r["peak"] == pytest.approx(629.3, abs=0.1)
    assert r["achieved"] == pytest.approx(72 * 256 ** 3 / 2.6e-3 / 1e9, rel=1e-3)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"], rel=1e-3)
    assert bench.fp64_issue(0.0, 1, 1.0) is None
    assert bench.fp64_issue(72.0, 1, 0.0) is None


def test_stage_bytes_are_the_algorithmic_totals():
    # 32 FP64 words per 3D cell-step, 21 per 2D cell-step
    assert sum(bench.STAGE_WORDS[3].values()) == 32
    assert sum(bench.STAGE_WORDS[2].values()) == 21


def test_roofline_block():
    stage = {k: 0.0 for k in bench.STAGES}
    stage.update(predictor=2.6, forward_x=0.8, spectral=1.8, inverse_x=0.6, correct=0.26)
    r = bench.roofline_block(3, "fp64", 256 ** 3, stage, 6660.6, "measured", sms=152, ghz=2.07)
    assert r["kernel"] == "k_predictor_tile" and r["bytes_per_cell"] == 104
    assert r["achieved"] == pytest.approx(104 * 256 ** 3 / 2.6e-3 / 1e9, rel=1e-3)
    assert r["frac"] == pytest.approx(r["achieved"] / 6660.6, rel=1e-3)
    assert r["traffic"] == int(99.6 * 256 ** 3) and "192^3" in r["traffic_source"]
    assert r["step_algorithmic_bytes_per_cell"] == 256
    m = bench.roofline_block(3, "mixed", 512 * 256 * 384, stage, 6660.6, "measured")
    assert m["kernel"] == "k_predictor_df_tile" and m["bytes_per_cell"] == 104
    assert m["traffic"] == int(100.4 * 512 * 256 * 384) and "256x128x192" in m["traffic_source"]
    d2 = bench.roofline_block(2, "fp64", 128 * 128, stage, 6660.6, "measured", sms=152, ghz=2.07)
    assert d2["bytes_per_cell"] == 72 and d2["step_algorithmic_bytes_per_cell"] == 168
    assert d2["kernel"] == "k_predictor<2>"


def test_measured_peaks_file_and_fallback(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.measured_peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6660.6}))
    assert bench.measured_peaks() == (6660.6, "measured")


def test_replica_throughput_is_whole_job():
    # N replicas of the same grid finishing within the slowest rank's time
    assert bench.replica_throughput(4, 1000, 10, 2.0) == pytest.approx(4 * 1000 * 10 / 2e-3 / 1e6)
