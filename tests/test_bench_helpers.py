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


class _BlockEngine:
    """Stand-in engine for BalancedBlocks: walker i costs (i + 1) cycles per sweep and 10 operator
    updates per sweep; walker `stops` stops (status 8) during block `stop_block`."""

    def __init__(self, n, stops=None, stop_block=None):
        self.st = {i: dict(sweeps=0, phase_cycles=[0, 0, 0, 0], slot_visits=0, worm_steps=0, status=0, L=100,
                           T=1.0, num_operators=40, worm_undos=0) for i in range(n)}
        self.stops, self.stop_block, self.blocks = stops, stop_block, 0

    def info(self, i):
        return dict(self.st[int(i)])

    def sweep_each(self, ids, ns, measure=True):
        from sse_gb300.engine import SSEError

        stopped = False
        for i, k in zip(ids.tolist(), ns.tolist()):
            if self.blocks == self.stop_block and i == self.stops:
                self.st[i]["status"] = 8
                stopped = True
                continue
            w = self.st[i]
            w["sweeps"] += k
            w["phase_cycles"][2] += k * (i + 1)
            w["slot_visits"] += 10 * k
        self.blocks += 1
        if stopped:
            raise SSEError(8, "worm cap")

    def last_timing(self):
        return 1.0, 1


def test_balanced_blocks_give_cheap_walkers_more_sweeps_and_count_stopped_ones(S):
    import numpy as np

    import bench

    eng = _BlockEngine(4, stops=2, stop_block=5)
    bb = bench.BalancedBlocks(eng, np.arange(4, dtype=np.int32))
    blocks, dev = bb.thermalise(5)
    # walker 0 costs a quarter of walker 3 per sweep: it gets four times the sweeps per block
    assert bb.k.tolist() == [4, 2, 1, 1] and blocks == 5 and all(eng.st[i]["sweeps"] == 5 for i in range(4))
    bb.reset_totals()
    done0 = {i: eng.st[i]["sweeps"] for i in range(4)}
    bb.block(measure=True)  # walker 2 stops in this block: the others finish, it leaves the set
    bb.block(measure=True)
    assert bb.stopped == 1 and bb.ids.tolist() == [0, 1, 3]
    assert bb.done_sw[2] == 0 and bb.done_ou[2] == 0.0
    for i in (0, 1, 3):
        assert bb.done_sw[i] == eng.st[i]["sweeps"] - done0[i] > 0
        assert bb.done_ou[i] == 10.0 * bb.done_sw[i]
