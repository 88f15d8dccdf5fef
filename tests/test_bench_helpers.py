"""Host helpers of bench.py: the roofline denominator and the algorithmic byte count."""

import io
import json

import pytest


def test_load_peaks_measured_and_fallback(monkeypatch):
    import bench

    monkeypatch.setattr(bench, "open", lambda *a, **k: io.StringIO(json.dumps({"hbm_gbs": 6663.9})), raising=False)
    assert bench.load_peaks() == (6663.9, "measured")

    def missing(*a, **k):
        raise FileNotFoundError

    monkeypatch.setattr(bench, "open", missing, raising=False)
    assert bench.load_peaks() == (6800.0, "fallback")


def test_walker_bytes_formula():
    import bench

    # diagonal r+w 4L, linking r 4L + w 16L, slot index 4L, worm 12 B per step, state 8 B per site
    assert bench.walker_bytes(1000, 500, 64) == 28 * 1000 + 12 * 500 + 8 * 64


def test_replica_streams_are_disjoint():
    import bench

    seen = set()
    for rank in range(4):
        s = set(bench.replica_streams(rank, 4096))
        assert len(s) == 4096 and not (s & seen)
        seen |= s
