"""bench.py's byte and FLOP models, on the host: the search's algorithmic bytes per candidate follow
the stamps and the geometry each interaction test reads, the roofline entries divide them by the
phase times, and the traffic table names its captures."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _conf(method, nPx=7, nPy=7, precision="mixed"):
    return {"approxBalls": {"method": method}, "precision": precision,
            "quadrature": {"outer": {"weights": [1.0] * nPx}, "inner": {"weights": [1.0] * nPy}}}


def test_search_bytes_per_candidate():
    # 16-bit stamp + vertex share (6 B), incidence entry (4 B), geometry of the test
    assert bench.search_bytes_per_candidate(_conf("retriangulate"), 2) == 6 + 4 + 48
    assert bench.search_bytes_per_candidate(_conf("baryCenter"), 2) == 6 + 4 + 16
    assert bench.search_bytes_per_candidate(_conf("baryCenter"), 3) == 6 + 4 + 24
    # other rules read the element's coordinates as double-float pairs
    assert bench.search_bytes_per_candidate(_conf("exactBall"), 2) == 6 + 4 + 48


def test_search_roofline_arithmetic(monkeypatch):
    monkeypatch.setattr(bench, "measured_peaks", lambda: {"hbm_gbs": 1000.0})
    st = {"ms_bfs": 10.0, "n_candidates": 1_000_000, "n_pairs": 500_000}
    r = bench.search_roofline(st, _conf("baryCenter"), 3)
    nbytes = 34 * 1_000_000 + 8 * 500_000
    assert r["algorithmic_bytes"] == nbytes and r["bytes_per_candidate"] == 34
    assert r["achieved"] == pytest.approx(nbytes / 0.010 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 1000.0)


def test_pass_traffic_table():
    for key, (per_pair, source) in bench.PASS_TRAFFIC.items():
        assert key in ("c2", "c4")
        assert 1.0 < per_pair < 64.0          # bytes per pair of the captured launch
        assert "k_pass" in source and "pairs" in source


def test_flop_model_counts_items():
    st = {"n_pairs": 100, "n_items_in": 500, "n_items_cut": 100, "n_subtri": 900}
    retri = bench.algorithmic_flops(st, _conf("retriangulate"), {"function": "constant"})
    assert retri == 100 * (12 + 7 * 87) + 500 * 10 + 100 * (133 + 26) + 400 * 84
    bary = bench.algorithmic_flops(st, _conf("baryCenter", nPx=11, nPy=11), {"function": "constant3D"})
    assert bary == 100 * 11 * 64 + 500 * 5
    # the general kernels count the inner-point loops
    par = bench.algorithmic_flops(st, _conf("retriangulate"), {"function": "parabola"})
    assert par == 100 * (12 + 7 * 198) + 900 * (11 + 7 * (51 + 7))
