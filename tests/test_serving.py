"""Host logic of the request loop (admission by projected memory, continuous batching,
retirement), against a fake engine: no GPU needed."""

import numpy as np


class FakeEngine:
    def __init__(self):
        self.next = 0
        self.walkers = {}
        self.models = 0
        self.calls = []

    def register_model(self, flat):
        self.models += 1
        return self.models - 1

    def create_walkers(self, mid, params):
        ids = np.arange(self.next, self.next + len(params), dtype=np.int32)
        self.next += len(params)
        for i, p in zip(ids.tolist(), params):
            self.walkers[i] = {"sweeps": 0, "p": p}
        return ids

    def init(self, ids):
        pass

    def sweep_each(self, ids, ns, measure=True):
        self.calls.append((list(ids), list(ns)))
        for i, n in zip(ids.tolist(), ns.tolist()):
            self.walkers[i]["sweeps"] += n

    def observables(self, ids):
        nobs = 16
        return [(np.full(nobs, float(self.walkers[i]["sweeps"])), np.ones(nobs, dtype=np.int64), np.zeros(nobs))
                for i in ids.tolist()]

    def info(self, i):
        return {"slot_visits": 10 * self.walkers[i]["sweeps"], "worm_steps": 5 * self.walkers[i]["sweeps"]}

    def destroy_walkers(self, ids):
        for i in ids.tolist():
            del self.walkers[i]


def test_continuous_batching_and_admission(S):
    from sse_gb300.serving import Request, ServingLoop, projected_walker_bytes

    eng = FakeEngine()
    reqs = [Request(k, 0.0, 0.5, "square", 4, 1.0, nwalkers=2 + k % 3, nsweeps=25 + 10 * k, seed=k) for k in range(6)]
    one = projected_walker_bytes(0.5, "square", 4, 1.0)
    loop = ServingLoop(eng, memory_budget=6 * one, tick_sweeps=10, clock=iter(np.arange(0, 1e6, 0.5)).__next__)
    res = loop.run(reqs, realtime=False)
    assert sorted(r.rid for r in res) == list(range(6))
    # every walker of every request ran exactly its sweep count
    for r in res:
        assert np.all(r.sums[:, 0] == reqs[r.rid].nsweeps)
    # admission never exceeded the budget when more than one request was active
    for ids, ns in eng.calls:
        assert len(ids) <= 6
        assert all(0 < n <= 10 for n in ns)
    # later requests joined launches while earlier ones were running
    assert any(len(set(ids)) > 2 for ids, _ in eng.calls)
    assert not eng.walkers  # all retired
    s = loop.summary()
    assert s["requests"] == 6 and s["p99_s"] >= s["p50_s"] > 0


def test_request_draw_distribution(S):
    from sse_gb300.serving import draw_requests

    reqs = draw_requests(7, 400, rate=200.0)
    gaps = np.diff([r.arrival for r in reqs])
    assert abs(gaps.mean() - 1 / 200) < 0.25 / 200
    assert {r.S for r in reqs} == {0.5, 1.0} and {r.lattice for r in reqs} == {"square", "bilayer"}
    assert all(8 <= r.side <= 64 and 0.5 <= r.beta <= 64 and 1 <= r.nwalkers <= 64 for r in reqs)
    assert all(1000 <= r.nsweeps <= 10000 for r in reqs)
    assert draw_requests(7, 5)[3] == draw_requests(7, 5)[3]


class CapStopEngine(FakeEngine):
    """Stops the walker of stream `stop_stream` once, at its `stop_at`-th sweep, like a worm that ran
    past the length cap (SSE_ERR_WORM_CAP)."""

    def __init__(self, stop_stream, stop_at):
        super().__init__()
        self.stop_stream, self.stop_at = stop_stream, stop_at
        self.status = {}

    def sweep_each(self, ids, ns, measure=True):
        from sse_gb300.engine import SSEError

        self.calls.append((list(ids), list(ns)))
        hit = False
        for i, n in zip(ids.tolist(), ns.tolist()):
            w = self.walkers[i]
            if self.status.get(i, 0):
                continue
            if w["p"]["stream"] == self.stop_stream and w["sweeps"] < self.stop_at <= w["sweeps"] + n:
                w["sweeps"] = self.stop_at
                self.status[i] = 8
                hit = True
            else:
                w["sweeps"] += n
        if hit:
            raise SSEError(8, "walker stopped with status 8")

    def info(self, i):
        d = super().info(i)
        d["status"] = self.status.get(i, 0)
        return d

    def create_walkers(self, mid, params):
        self.created = getattr(self, "created", []) + [p["stream"] for p in params]
        return super().create_walkers(mid, params)


def test_stopped_walker_is_replaced_by_a_fresh_chain(S):
    from sse_gb300.serving import Request, ServingLoop

    eng = CapStopEngine(stop_stream=1, stop_at=17)
    req = Request(0, 0.0, 1.0, "square", 4, 1.0, nwalkers=3, nsweeps=40, seed=5)
    loop = ServingLoop(eng, memory_budget=10**12, tick_sweeps=10, clock=iter(np.arange(0, 1e6, 0.5)).__next__)
    (res,) = loop.run([req], realtime=False)
    assert res.status == "ok" and res.replaced == 1
    # slot 1's replacement ran stream 1 + 1*3 = 4 for all 40 sweeps, from init!
    assert eng.created == [0, 1, 2, 4]
    assert not eng.walkers  # all retired
    assert np.all(res.sums[:, 0] == 40)
    assert res.operator_updates == 3 * 40 * 15 + 17 * 15  # the stopped walker's work is counted too
    assert loop.summary()["walkers_replaced"] == 1


def test_request_fails_when_replacements_are_used_up(S):
    from sse_gb300.serving import Request, ServingLoop

    eng = CapStopEngine(stop_stream=0, stop_at=3)
    req = Request(0, 0.0, 1.0, "square", 4, 1.0, nwalkers=2, nsweeps=20, seed=5)
    loop = ServingLoop(eng, memory_budget=10**12, tick_sweeps=10, retries=0,
                       clock=iter(np.arange(0, 1e6, 0.5)).__next__)
    (res,) = loop.run([req], realtime=False)
    assert res.status == "SSE_ERR_WORM_CAP" and res.replaced == 0
    assert loop.summary()["failed"] == 1


def test_cost_aware_ticks_give_small_walkers_more_sweeps(S):
    """With tick_seconds every walker gets as many sweeps per tick as fit the tick at the estimated
    rate, so a small model's walkers run many more sweeps per launch than a large model's."""
    from sse_gb300.serving import Request, ServingLoop, projected_sweep_cost

    eng = FakeEngine()
    small = Request(0, 0.0, 0.5, "square", 4, 1.0, nwalkers=2, nsweeps=400, seed=1)
    large = Request(1, 0.0, 1.0, "bilayer", 16, 8.0, nwalkers=2, nsweeps=400, seed=2)
    loop = ServingLoop(eng, memory_budget=10**12, tick_seconds=0.25, walker_rate=1e6,
                       clock=iter(np.arange(0, 1e6, 0.5)).__next__)
    res = loop.run([small, large], realtime=False)
    assert sorted(r.rid for r in res) == [0, 1]
    ids, ns = eng.calls[0]
    k_small, k_large = ns[0], ns[2]
    c_small = projected_sweep_cost(0.5, "square", 4, 1.0)
    c_large = projected_sweep_cost(1.0, "bilayer", 16, 8.0)
    assert k_small == min(400, int(0.25 * 1e6 / c_small)) and k_large == max(1, int(0.25 * 1e6 / c_large))
    assert k_small > k_large
    # the rate estimate moved towards the measured one after the first tick
    assert loop.rate != 1e6
    for r in res:
        assert np.all(r.sums[:, 0] == 400)


def test_admission_refuses_requests_over_the_projected_time_budget(S):
    """With max_request_seconds, a request whose projected device time exceeds it is refused at
    admission (counted, never run); the others run as usual."""
    from sse_gb300.serving import Request, ServingLoop, projected_request_seconds

    eng = FakeEngine()
    small = Request(0, 0.0, 0.5, "square", 8, 1.0, nwalkers=2, nsweeps=10, seed=1)
    big = Request(1, 0.0, 1.0, "bilayer", 64, 8.0, nwalkers=4, nsweeps=10, seed=2)
    assert projected_request_seconds(small) < 1.0 < 60.0 < projected_request_seconds(big)
    loop = ServingLoop(eng, memory_budget=1 << 40, tick_sweeps=10, clock=iter(np.arange(0, 1e6, 0.5)).__next__,
                       max_request_seconds=60.0)
    res = loop.run([small, big], realtime=False)
    assert [r.rid for r in res] == [0] and loop.refused == [1]
    assert loop.summary()["refused"] == 1
    assert all(len(ids) == 2 for ids, _ in eng.calls)  # the big request's walkers were never created
