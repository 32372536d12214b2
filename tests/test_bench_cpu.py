"""Host logic of bench.py that feeds the top-level JSON keys, on CPU: which
serving rate `serving_p99_ms_1024` is quoted at, and the roofline's DRAM
traffic lookup from the committed ncu summary."""
from __future__ import annotations

import importlib.util
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)  # module level: constants and functions only
    return mod


def _rate(offered, pairs, p99):
    return {"offered_per_s": offered, "pairs_per_s": pairs, "p99_ms_1024": p99}


def test_serving_p99_is_quoted_at_the_highest_unsaturated_rate():
    b = _bench()
    serving = {"modes": {"direct": {"rates": [
        _rate(1000, [1001.0, 998.0, 1003.0], [0.15, 0.19, 0.17]),
        _rate(20000, [20100.0, 19500.0, 20300.0], [0.63, 0.88, 0.76]),
        _rate(50000, [28000.0, 27600.0, 28100.0], [31.8, 32.4, 32.2]),  # saturated
    ]}}}
    # the worst repeat at 20k: 50k did not keep up with its offer
    assert b.serving_p99_1024(serving) == (0.88, 20000)
    # a rate that kept up in two repeats but not the third is saturated
    serving["modes"]["direct"]["rates"][1]["pairs_per_s"][1] = 18000.0
    assert b.serving_p99_1024(serving) == (0.19, 1000)
    assert b.serving_p99_1024(serving, mode="copy") == (None, None)
    assert b.serving_p99_1024(None) == (None, None)


def test_traffic_lookup_matches_committed_profile():
    b = _bench()
    lines = (ROOT / "profiles" / "traffic_per_launch.txt").read_text().splitlines()
    assert lines, "the committed traffic summary is empty"
    for line in lines:
        key, value = line.rsplit(None, 1)
        assert b.traffic_per_launch(key) == float(value)
    assert b.traffic_per_launch("no such kernel") is None
    # the headline's kernel name as bench.py builds it, at the lags the autotuner picks
    for lag in (4, 5):
        assert b.traffic_per_launch(f"fft_batch_ws<3,2>x64 lag{lag}") is not None
