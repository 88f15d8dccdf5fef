"""Request loop with continuous batching over the GPU engine.

A request asks for `nwalkers` independent chains of one model (S=1/2 or S=1
Heisenberg on a square lattice or a square bilayer) at inverse temperature
`beta` for `nsweeps` Carlo steps (the first `thermalization` of them
unmeasured).  The loop

* admits pending requests in arrival order while the projected opstring memory
  of all admitted walkers stays within `memory_budget` bytes,
* keeps every admitted walker resident on the device,
* advances all active walkers together, each by min(tick, remaining) sweeps,
  in one persistent launch per tick (`sse_sweep_each`), so requests that
  arrive while others run join the next launch,
* retires a request as soon as its walkers are done, reporting its
  observables and its time-to-result (completion - arrival),
* refuses, when given a bound, a request whose projected device time exceeds it,
* replaces a walker that the engine stopped (a worm past the step cap,
  SSE_ERR_WORM_CAP) with a fresh chain, up to `retries` times per walker:
  slot k of a request runs stream k, its a-th replacement stream
  k + a * nwalkers, each replacement all of the request's sweeps from
  init!; with retries exhausted the request is reported as failed.

A walker's trajectory depends only on its own (seed, stream), so a request's
result is the same whether it runs alone or mixed with others.
"""

from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from .engine import STATUS_NAMES, SSEError
from .lattice import UnitCells
from .magnet import MagnetModel
from .tables import flatten_model


@dataclass
class Request:
    rid: int
    arrival: float  # seconds after the start of the run
    S: float  # 0.5 or 1.0
    lattice: str  # "square" or "bilayer"
    side: int
    beta: float
    nwalkers: int
    nsweeps: int
    seed: int
    thermalization: int = 0

    @property
    def model_key(self):
        return (self.S, self.lattice, self.side)


@dataclass
class Result:
    rid: int
    arrival: float
    finish: float
    names: list
    sums: np.ndarray  # [nwalkers, nobs]
    counts: np.ndarray
    operator_updates: int = 0
    energy: float = float("nan")
    status: str = "ok"  # or the sse_status name that stopped one of its walkers
    replaced: int = 0  # walkers replaced by a fresh chain after the engine stopped them
    undone: int = 0  # thermalisation sweeps whose worm phase was undone at the worm step cap

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


def model_params(S: float, lattice: str, side: int) -> dict:
    """Heisenberg J=1; the bilayer adds a rung coupling J_perp = 0.5."""
    if lattice == "square":
        return {"lattice": {"unitcell": UnitCells.square, "size": (side, side)}, "J": 1.0, "S": S,
                "measure": ["magnetization", "staggered_magnetization"]}
    if lattice == "bilayer":
        return {"lattice": {"unitcell": UnitCells.square_bilayer, "size": (side, side)}, "S": S, "J": 1.0, "Jp": 0.5,
                "parameter_map": {"J": ["Jp", "J", "J", "J", "J"]}, "measure": ["magnetization"]}
    raise ValueError(f"unknown lattice {lattice}")


def projected_operators(S: float, lattice: str, side: int, beta: float) -> float:
    """Expected operator count n ~ beta * bonds * (energy offset + bond energy) per bond."""
    nbonds = side * side * (5 if lattice == "bilayer" else 2)
    per_bond = 0.75 if S == 0.5 else 2.6
    return beta * nbonds * per_bond


def projected_slots(S: float, lattice: str, side: int, beta: float) -> int:
    """Opstring capacity to reserve: 1.3 x a cutoff of about 2.2 n."""
    return int(1.3 * (2.2 * projected_operators(S, lattice, side, beta) + 100)) + 64


def projected_walker_bytes(S: float, lattice: str, side: int, beta: float) -> int:
    """Device bytes a walker is expected to reserve: 40 B per opstring slot (opcode, 32-byte record,
    slot index) plus per-site arrays."""
    nsites = side * side * (2 if lattice == "bilayer" else 1)
    return int(40 * projected_slots(S, lattice, side, beta) + 16 * nsites + 4096)


def projected_sweep_cost(S: float, lattice: str, side: int, beta: float) -> float:
    """Operator-updates per sweep: about L + W = 2.2 n + 2 n."""
    return 4.2 * projected_operators(S, lattice, side, beta) + 100


def projected_request_seconds(req, step_seconds: float = 1.2e-6) -> float:
    """Device seconds one walker of `req` is projected to need, bounded from the expensive side.

    A fresh walker runs the reference's worm-count controller transient (src/sse.jl:204-217): the
    average worm length starts at 1 and rises by 1 % per sweep, so every sweep runs far more worm
    steps than the equilibrium 2n.  On the oracle, 64x64 S=1/2 at beta = 64 ran 35-55 x 2n steps per
    sweep over its first 30 sweeps, the 48x48 S=1 bilayer at beta = 4 and 16 ran 60-145 x 2n.  Its
    operator count meanwhile grows with the cutoff: about 10-30 N T after Carlo.init!'s diagonal
    sweeps, then about 1.5x per sweep up to the equilibrium n.  The projection takes sweep k to hold
    min(n_eq, 15 N T 1.5^k) operators and to run 100 (S=1/2) or 260 (S=1) worm steps per operator,
    each a dependent step of `step_seconds` (one warp chases one walker; about 1.2 us at full load)."""
    n_eq = projected_operators(req.S, req.lattice, req.side, req.beta)
    nsites = req.side * req.side * (2 if req.lattice == "bilayer" else 1)
    per_op = 100.0 if req.S == 0.5 else 260.0
    total = 0.0
    for k in range(req.nsweeps):
        n_k = min(n_eq, 15.0 * nsites / req.beta * 1.5 ** k)
        total += per_op * n_k
        if n_k >= n_eq:
            total += per_op * n_eq * (req.nsweeps - k - 1)
            break
    return total * step_seconds


def draw_requests(seed: int, count: int, rate: float = 200.0, side=(8, 64), beta=(0.5, 64.0), walkers=(1, 64),
                  sweeps=(1000, 10000), therm_fraction: float = 0.2, sweep_scale: float = 1.0):
    """Poisson arrivals (mean `rate` per second) with the request distribution of the serving workload:
    S in {1/2, 1}, square or bilayer, side uniform, beta and sweeps log-uniform, walkers uniform.
    `sweep_scale` multiplies every drawn sweep count (at least 1 sweep remains), so that a bounded
    run can keep the distribution's shape."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(count):
        t += rng.exponential(1.0 / rate)
        S = float(rng.choice([0.5, 1.0]))
        lat = str(rng.choice(["square", "bilayer"]))
        sd = int(rng.integers(side[0], side[1] + 1))
        b = float(math.exp(rng.uniform(math.log(beta[0]), math.log(beta[1]))))
        nw = int(rng.integers(walkers[0], walkers[1] + 1))
        ns = max(1, int(round(sweep_scale * math.exp(rng.uniform(math.log(sweeps[0]), math.log(sweeps[1]))))))
        out.append(Request(rid, t, S, lat, sd, b, nw, ns, seed=int(rng.integers(0, 2**62)),
                           thermalization=int(therm_fraction * ns)))
    return out


@dataclass
class _Active:
    req: Request
    ids: np.ndarray
    done: np.ndarray  # sweeps done, per walker
    nbytes: int = 0
    cost: float = 1.0  # projected operator-updates per sweep of one walker
    attempts: np.ndarray = None  # replacements so far, per walker slot
    replaced: int = 0
    spent_updates: int = 0  # operator-updates of walkers that were replaced


class ServingLoop:
    """Continuous batching.  With `tick_seconds` set, every walker gets as many sweeps per tick as
    fit in that time at the estimated per-walker rate (operator-updates/s, re-estimated from each
    tick), so small requests finish in one tick instead of waiting for the largest walker; without
    it every walker gets `tick_sweeps` sweeps per tick."""

    def __init__(self, engine, memory_budget: int, tick_sweeps: int = 10, clock=time.perf_counter,
                 tick_seconds: float | None = None, walker_rate: float = 1.5e6, retries: int = 2,
                 max_request_seconds: float | None = None):
        """`max_request_seconds`: refuse, at admission, a request whose projected device time
        (projected_request_seconds) exceeds it: a kernel cannot be interrupted inside a sweep, so one
        admitted request whose sweeps take minutes would stall every request batched with it."""
        self.eng = engine
        self.max_request_seconds = max_request_seconds
        self.refused: list = []
        self.retries = int(retries)
        self.budget = int(memory_budget)
        self.tick = int(tick_sweeps)
        self.tick_seconds = tick_seconds
        self.rate = float(walker_rate)
        self.clock = clock
        self.models: dict = {}
        self.pending: list = []
        self.active: list = []
        self.results: list = []
        self.used = 0
        self.t0 = None
        self.launches = 0

    def _model(self, key):
        if key not in self.models:
            S, lat, side = key
            flat = flatten_model(MagnetModel(model_params(S, lat, side)))
            self.models[key] = (self.eng.register_model(flat), flat)
        return self.models[key]

    def now(self) -> float:
        return self.clock() - self.t0

    def submit(self, req: Request):
        self.pending.append(req)

    def admit(self):
        """Admit pending requests in arrival order while the projected memory fits."""
        admitted = []
        while self.pending:
            req = self.pending[0]
            if self.max_request_seconds is not None and projected_request_seconds(req) > self.max_request_seconds:
                self.pending.pop(0)
                self.refused.append(req.rid)
                continue
            need = req.nwalkers * projected_walker_bytes(req.S, req.lattice, req.side, req.beta)
            if self.active and self.used + need > self.budget:
                break
            self.pending.pop(0)
            ids = self._new_walkers(req, list(range(req.nwalkers)))
            cost = projected_sweep_cost(req.S, req.lattice, req.side, req.beta)
            self.active.append(_Active(req, ids, np.zeros(req.nwalkers, dtype=np.int64), need, cost,
                                       np.zeros(req.nwalkers, dtype=np.int64)))
            self.used += need
            admitted.append(req.rid)
        return admitted

    def _new_walkers(self, req: Request, streams):
        mid, flat = self._model(req.model_key)
        params = [dict(T=1.0 / req.beta, seed=req.seed, stream=int(k), thermalization=req.thermalization)
                  for k in streams]
        ids = self.eng.create_walkers(mid, params)
        if hasattr(self.eng, "reserve"):
            self.eng.reserve(ids, projected_slots(req.S, req.lattice, req.side, req.beta))
        self.eng.init(ids)
        return np.asarray(ids, dtype=np.int32)

    def step(self):
        """One tick: every active walker advances min(tick, remaining) sweeps in one launch."""
        if not self.active:
            return []
        ids, ns = [], []
        planned = 0.0
        for a in self.active:
            left = a.req.nsweeps - a.done
            if self.tick_seconds:
                k = np.maximum(1, np.minimum(left, int(max(1, self.tick_seconds * self.rate / a.cost))))
            else:
                k = np.minimum(self.tick, left)
            k = np.where(left > 0, k, 0)
            planned = max(planned, float(k.max()) * a.cost)
            ids.append(a.ids)
            ns.append(k.astype(np.int32))
            a.done += k
        failed = {}
        t_start = self.clock()
        try:
            self.eng.sweep_each(np.concatenate(ids), np.concatenate(ns), measure=True)
        except SSEError as err:
            # every other walker finished its sweeps; replace the walkers that stopped, or fail
            # their request when its replacements are used up
            stopped = 0
            for a in self.active:
                for slot, i in enumerate(a.ids.tolist()):
                    st = self.eng.info(i)["status"]
                    if st == 0:
                        continue
                    stopped += 1
                    if a.attempts[slot] < self.retries:
                        a.attempts[slot] += 1
                        inf = self.eng.info(i)
                        a.spent_updates += inf["slot_visits"] + inf["worm_steps"]
                        self.eng.destroy_walkers(np.array([i], dtype=np.int32))
                        stream = slot + int(a.attempts[slot]) * a.req.nwalkers
                        a.ids[slot] = self._new_walkers(a.req, [stream])[0]
                        a.done[slot] = 0
                        a.replaced += 1
                    else:
                        failed[a.req.rid] = STATUS_NAMES.get(st, str(st))
            if not stopped:
                raise err
        self.launches += 1
        took = self.clock() - t_start
        if self.tick_seconds and took > 0 and planned > 0:
            self.rate = 0.7 * self.rate + 0.3 * (planned / took)
        finished = []
        still = []
        for a in self.active:
            if (a.done >= a.req.nsweeps).all() or a.req.rid in failed:
                finished.append(a)
            else:
                still.append(a)
        self.active = still
        out = []
        t = self.now()
        for a in finished:
            obs = self.eng.observables(a.ids)
            sums = np.array([o[0] for o in obs])
            counts = np.array([o[1] for o in obs])
            ou = a.spent_updates
            undone = 0
            for i in a.ids.tolist():
                inf = self.eng.info(i)
                ou += inf["slot_visits"] + inf["worm_steps"]
                undone += inf.get("worm_undos", 0)
            self.eng.destroy_walkers(a.ids)
            self.used -= a.nbytes
            mid, flat = self._model(a.req.model_key)
            from .engine import observable_names

            names = observable_names(flat.est_prefixes)
            s = sums.sum(0)
            c = counts.sum(0)
            energy = (s[4] / c[4]) / (s[0] / c[0]) if (c[0] and c[4] and s[0]) else float("nan")
            res = Result(a.req.rid, a.req.arrival, t, names, sums, counts, ou, energy,
                         status=failed.get(a.req.rid, "ok"), replaced=a.replaced, undone=undone)
            self.results.append(res)
            out.append(res)
        return out

    def run(self, requests, realtime: bool = True, max_seconds: float = float("inf")):
        """Feed `requests` by arrival time (sleeping while idle when `realtime`) until all are done."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        self.t0 = self.clock()
        i = 0
        while i < len(reqs) or self.pending or self.active:
            t = self.now()
            if t > max_seconds:
                break
            while i < len(reqs) and (reqs[i].arrival <= t or not realtime):
                self.submit(reqs[i])
                i += 1
            self.admit()
            if self.active:
                self.step()
            elif i < len(reqs) and realtime:
                time.sleep(max(0.0, min(0.05, reqs[i].arrival - self.now())))
        return self.results

    def summary(self):
        lat = np.array([r.latency for r in self.results])
        ou = sum(r.operator_updates for r in self.results)
        span = max((r.finish for r in self.results), default=0.0)
        return {
            "requests": len(self.results),
            "refused": len(self.refused),
            "failed": sum(r.status != "ok" for r in self.results),
            "walkers_replaced": sum(r.replaced for r in self.results),
            "thermalisation_sweeps_undone": sum(r.undone for r in self.results),
            "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "mean_s": float(lat.mean()) if len(lat) else None,
            "operator_updates_per_s": ou / span if span > 0 else None,
            "makespan_s": span,
            "launches": self.launches,
        }
