"""Benchmark: batched SSE sweeps on GB300.

Workload (the batched uniform configuration): 4096 independent walkers of the
S=1/2 antiferromagnetic Heisenberg model on a 32x32 periodic square lattice
(2048 bonds) at beta = 16, per-walker Philox streams, 2000 thermalisation
sweeps, then measured sweeps (Carlo.sweep! + Carlo.measure!).  A "step" is
one sweep block: `--sweeps-per-step` Carlo steps of every walker in one
persistent launch.  Inputs are synthetic (generated models, seeded chains).

  python bench.py [--gpus N] [--steps K] [--warmup W]
  python bench.py --impl reference     # the CPU implementation of the path on the host cores

Prints one JSON line.  `value` is whole-job walker-sweeps/s from CUDA events
around the sweep launches (walker state resident in HBM); `e2e` is the same
metric through the public API per step (ids H2D, sweep, observables D2H),
wall-clock.  `roofline` relates the algorithmic bytes of the sweep kernel
(28 L + 12 W + 8 N per walker-sweep) to the measured HBM copy bandwidth.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import _sse_loader  # noqa: E402

METRIC = "walker-sweeps/s"


def workload_name(args):
    """The headline workload with the sizes this run uses; the defaults give "4096 walkers, S=1/2
    Heisenberg, 32x32 periodic square (2048 bonds), beta=16"."""
    return (f"{args.walkers} walkers, S=1/2 Heisenberg, {args.side}x{args.side} periodic square "
            f"({2 * args.side * args.side} bonds), beta={args.beta:g}")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--walkers", type=int, default=4096)
    ap.add_argument("--side", type=int, default=32)
    ap.add_argument("--beta", type=float, default=16.0)
    ap.add_argument("--therm", type=int, default=2000, help="thermalisation sweeps before the warm-up steps")
    ap.add_argument("--sweeps-per-step", type=int, default=50)
    ap.add_argument("--plain-walkers", type=int, default=8)
    ap.add_argument("--wpb", type=int, default=0,
                    help="walkers (warps) per block of the sweep launch, staging off; 0: the autotuner chooses")
    ap.add_argument("--cpu-sweeps", type=int, default=2000,
                    help="sweeps per chain in the CPU baseline sample (about 10 s on 16 cores for the default workload)")
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--uneven-therm", type=int, default=150,
                    help="thermalisation sweeps per walker of the uneven batch (worm-count controller active)")
    ap.add_argument("--profile", action="store_true", help="open a profiler range around the timed steps only")
    ap.add_argument("--serving-requests", type=int, default=200, help="requests in the serving run (0: skip)")
    ap.add_argument("--serving-sweep-scale", type=float, default=1e-3,
                    help="--workload serving: factor on the drawn 10^3-10^4 sweeps per request")
    ap.add_argument("--serving-max-seconds", type=float, default=1200.0,
                    help="--workload serving: stop admitting requests after this many seconds")
    ap.add_argument("--serving-request-budget", type=float, default=60.0,
                    help="--workload serving: refuse a request whose projected device time exceeds this")
    ap.add_argument("--workload", default="uniform",
                    choices=["uniform", "single", "uneven", "bilayer", "serving", "magnet_bench", "cluster_bench"],
                    help="uniform: the headline batch; single: one 8x8 walker at beta=2; uneven: 8192 walkers of "
                         "mixed sizes and temperatures; bilayer: 2048 S=1 bilayer walkers 48x48; serving: the request loop over "
                         "the serving distribution's full side and beta ranges; magnet_bench / "
                         "cluster_bench: the reference's own whole-job benchmark tasks, batched")
    return ap.parse_args()


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_model(S, side):
    return S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (side, side)}, "J": 1.0,
                          "measure": ["magnetization", "staggered_magnetization"]})


def walker_bytes(L, W, N):
    """Algorithmic DRAM bytes of one walker-sweep: diagonal update r+w 4L, linking r 4L + w 16L (the
    compacted records), 4L of slot bookkeeping (the chunk index and writing the operators' final codes
    back), worm 12 B per step (link r, opcode r+w), state r+w 4N+4N."""
    return 28.0 * L + 12.0 * W + 8.0 * N


def dist_setup(args):
    rank, world, local = 0, 1, 0
    if "RANK" in os.environ and int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist

        rank = int(os.environ["RANK"])
        world = int(os.environ["WORLD_SIZE"])
        local = int(os.environ.get("LOCAL_RANK", rank))
        dist.init_process_group("gloo")
    return rank, world, local


def replica_streams(rank, nwalkers):
    """Walker ids (Philox streams) of one replica: rank r runs streams r*n .. r*n + n - 1, so the
    replicas of a multi-GPU run are disjoint sets of independent chains (no data exchange)."""
    return range(rank * nwalkers, (rank + 1) * nwalkers)


def barrier_max(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier_sum(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def cpu_baseline(S, flat, states, args, nthreads):
    """The CPU restatement (oracle) timed on the host cores, one chain per thread, started from
    GPU-thermalised walker states so that it runs the same opstring lengths."""
    from oracle import oracle as O

    om = O.OracleModel(flat)
    walkers = []
    for k, (ops, st, inf) in enumerate(states[:nthreads]):
        w = O.OracleWalker(om, T=1.0 / args.beta, seed=args.seed, stream=k, thermalization=0)
        w.set_opstring(ops, inf["num_operators"])
        w.set_state(st)
        w.w.ctr = inf["rng_counter"]
        w.w.num_worms = inf["num_worms"]
        w.w.avg_worm_length = inf["avg_worm_length"]
        w.w.sweeps = 1
        walkers.append(w)
    t0 = time.perf_counter()
    O.run_parallel(om, walkers, args.cpu_sweeps, measure=True, nthreads=nthreads)
    dt = time.perf_counter() - t0
    ws = len(walkers) * args.cpu_sweeps
    steps = sum(w.w.worm_steps_total for w in walkers)
    slots = sum(w.w.slot_visits_total for w in walkers)
    return {
        "value": ws / dt,
        "unit": METRIC,
        "cores": nthreads,
        "kind": "port",
        "sample": f"{len(walkers)} chains x {args.cpu_sweeps} measured sweeps of the same workload from GPU-thermalised states, one chain per host thread",
        "operator_updates_per_s": (steps + slots) / dt,
        "seconds": dt,
    }


def parity_check(S, flat, eng, ids, states, args, nsweeps=5):
    """The benchmarked walkers continued on both sides: `states` were exported after the timed
    region; the same walkers run `nsweeps` more Carlo steps on the GPU and, imported, in the oracle.
    Opstrings, spin states, cutoffs, replay counters and controller doubles must be equal bit for
    bit, the observables of those sweeps within 1e-12 relative."""
    from oracle import oracle as O

    om = O.OracleModel(flat)
    chains = []
    for k, (ops, st, inf) in enumerate(states):
        w = O.OracleWalker(om, T=1.0 / args.beta, seed=args.seed, stream=k, thermalization=args.therm)
        w.set_opstring(ops, inf["num_operators"])
        w.set_state(st)
        w.w.ctr = inf["rng_counter"]
        w.w.num_worms = inf["num_worms"]
        w.w.avg_worm_length = inf["avg_worm_length"]
        w.w.sweeps = inf["sweeps"]
        chains.append(w)
    sub = np.ascontiguousarray(ids[: len(states)], dtype=np.int32)
    eng.observables(sub, reset=True)
    eng.sweep(sub, nsweeps, measure=True)
    O.run_parallel(om, chains, nsweeps, measure=True, nthreads=min(len(chains), os.cpu_count() or 1))
    bad, worst = [], 0.0
    for wid, w in zip(sub.tolist(), chains):
        ops, st, inf = eng.export(wid)
        same = (inf["status"] == w.w.status == 0 and inf["L"] == w.w.L and inf["rng_counter"] == w.w.ctr
                and inf["num_operators"] == w.w.num_operators and inf["num_worms"] == w.w.num_worms
                and inf["avg_worm_length"] == w.w.avg_worm_length and np.array_equal(ops, w.ops)
                and np.array_equal(st, w.state))
        s, c, _ = eng.observables([wid])[0]
        so, co, _ = w.obs()
        rel = float(np.max(np.abs(s - so) / np.maximum(np.abs(so), 1e-300))) if len(so) else 0.0
        worst = max(worst, rel)
        if not same or not np.array_equal(c, co) or rel > 1e-12:
            bad.append(wid)
    return {"walkers": len(chains), "sweeps": nsweeps, "bit_exact_walkers": len(chains) - len(bad),
            "max_rel_observable_diff": worst, "mismatched_walkers": bad,
            "what": "exported after the timed region, continued on the GPU and in the oracle; opstring, state, "
                    "cutoff, replay counter and controller compared bit for bit, observables to 1e-12"}


def run_serving(args, device, full=False):
    """The request loop: Poisson arrivals at 200 requests/s, continuous batching, p50/p99 time-to-result.

    full=False (the default benchmark's serving block): the serving workload's distribution scaled
    so that the run takes about a minute -- side 8-24, beta 0.5-4 and 20-200 sweeps (log-uniform),
    1-64 walkers, S=1/2 or 1, square or bilayer.

    full=True (`--workload serving`): the distribution's own ranges -- side 8-64, beta 0.5-64
    log-uniform, 1-64 walkers, S=1/2 or 1, square or bilayer -- with the drawn 10^3-10^4 sweeps
    multiplied by `--serving-sweep-scale` (default 1/1000, so 1-10 sweeps), because a single S=1
    64x64 bilayer walker at beta = 64 needs seconds per sweep (L near 7.5 million slots) and the
    drawn counts would take hours.  Requests whose projected device time (the worm-count controller's
    transient included, serving.projected_request_seconds) exceeds `--serving-request-budget` are
    refused at admission and counted; the loop stops at `--serving-max-seconds`; the line says how many
    requests completed."""
    from sse_gb300.engine import Engine
    from sse_gb300.serving import ServingLoop, draw_requests

    if full:
        nreq = args.serving_requests
        reqs = draw_requests(args.seed, nreq, rate=200.0, side=(8, 64), beta=(0.5, 64.0), walkers=(1, 64),
                             sweeps=(1000, 10000), sweep_scale=args.serving_sweep_scale)
        budget = 180 << 30
        dist = (f"side 8-64, beta 0.5-64 log-uniform, 1-64 walkers, S in {{1/2,1}}, square or bilayer (J_perp=0.5), "
                f"10^3-10^4 sweeps log-uniform x {args.serving_sweep_scale:g} (at least 1), 20% thermalisation; "
                f"requests projected over {args.serving_request_budget:g} s of device time refused at admission")
    else:
        nreq = args.serving_requests
        reqs = draw_requests(args.seed, nreq, rate=200.0, side=(8, 24), beta=(0.5, 4.0),
                             walkers=(1, 64), sweeps=(20, 200))
        budget = 40 << 30
        dist = ("side 8-24, beta 0.5-4 and sweeps 20-200 log-uniform, 1-64 walkers, S in {1/2,1}, square or bilayer "
                "(J_perp=0.5), 20% thermalisation")
    eng = Engine(device)
    loop = ServingLoop(eng, memory_budget=budget, tick_seconds=0.25,
                       max_request_seconds=args.serving_request_budget if full else None)
    # warm the model cache (table builds are host work outside the request path)
    for r in reqs:
        loop._model(r.model_key)
    t0 = time.perf_counter()
    loop.run(reqs, realtime=True, max_seconds=args.serving_max_seconds if full else float("inf"))
    wall = time.perf_counter() - t0
    out = loop.summary()
    eng.close()
    done = {r.rid for r in loop.results}
    out.update(rate_per_s=200.0, requests_drawn=nreq, requests_completed=len(done), wall_seconds=wall,
               distribution=dist + "; 0.25 s ticks with per-walker sweep counts sized by projected cost",
               memory_budget_gb=budget >> 30)
    if full and loop.results:
        # the completed request with the most projected work per sweep, and its time-to-result
        byid = {r.rid: r for r in reqs}
        r, lat = max(((byid[x.rid], x.latency) for x in loop.results),
                     key=lambda t: t[0].side ** 2 * t[0].beta * (2 if t[0].lattice == "bilayer" else 1) * t[0].S)
        out["largest_completed"] = {"S": r.S, "lattice": r.lattice, "side": r.side, "beta": round(r.beta, 2),
                                    "walkers": r.nwalkers, "sweeps": r.nsweeps, "time_to_result_s": round(lat, 2)}
    return out


def run_reference(args):
    """--impl reference: the CPU implementation of the path (the oracle restatement of the
    reference's sweep; Julia is not available to run the reference itself) on all host cores."""
    rank, world, _ = dist_setup(args)
    if rank != 0:
        return
    S = _sse_loader.load()
    from oracle import oracle as O

    flat = S.flatten_model(make_model(S, args.side))
    om = O.OracleModel(flat)
    nthreads = args.cpu_threads or os.cpu_count() or 1
    walkers = [O.OracleWalker(om, T=1.0 / args.beta, seed=args.seed, stream=k, thermalization=10**9) for k in range(nthreads)]
    for w in walkers:
        w.init()
    # bounded thermalisation: opstring lengths and worm counts near their working values
    O.run_parallel(om, walkers, 300, measure=False, nthreads=nthreads)
    for w in walkers:
        w.w.thermalization = 0
    per_step = max(1, args.cpu_sweeps // 4)
    for _ in range(args.warmup):
        O.run_parallel(om, walkers, per_step, measure=True, nthreads=nthreads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.run_parallel(om, walkers, per_step, measure=True, nthreads=nthreads)
    dt = time.perf_counter() - t0
    value = len(walkers) * per_step * args.steps / dt
    line = {
        "impl": "reference",
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "i32+f64", "data": "synthetic",
        "config": {"workload": workload_name(args), "walkers_per_step": len(walkers), "sweeps_per_step": per_step,
                   "note": "CPU restatement of the reference sweep (Julia reference not runnable here)"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": nthreads, "kind": "port",
                         "sample": f"{len(walkers)} chains x {per_step} sweeps per step after 300 thermalisation sweeps"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def sweep_tolerant(eng, ids, nsweeps, measure=True, graph=False):
    """sse_sweep over a batch; walkers stopped by an error (a worm past the step cap) are dropped
    from the batch and counted, the others continue."""
    from sse_gb300.engine import SSEError

    try:
        eng.sweep(ids, nsweeps, measure=measure, graph=graph)
        return ids, 0
    except SSEError:
        ok = np.array([i for i in ids.tolist() if eng.info(i)["status"] == 0], dtype=np.int32)
        return ok, len(ids) - len(ok)


def run_other_workload(args):
    """The other configurations, each printed as its own JSON line (not the headline line)."""
    S = _sse_loader.load()
    from sse_gb300.engine import Engine

    eng = Engine(0)
    rng = np.random.default_rng(args.seed)
    line = {"workload": args.workload}
    if args.workload == "single":
        # one walker, 8x8 S=1/2 Heisenberg, beta=2: persistent launch vs one launch per sweep vs the CPU oracle
        from oracle import oracle as O

        flat = S.flatten_model(make_model(S, 8))
        mid = eng.register_model(flat)
        # 2000 thermalisation sweeps, then every timed sweep runs measure! (GPU and CPU alike)
        a, b = eng.create_walkers(mid, [dict(T=0.5, seed=args.seed, stream=0, thermalization=2000)] * 2)
        eng.init([a, b])
        eng.sweep([a, b], 2000, measure=False)
        n = 20000
        c0 = np.array(eng.info(int(a))["phase_cycles"], dtype=float)
        eng.sweep([a], n, measure=True)
        ms, _ = eng.last_timing()
        c1 = np.array(eng.info(int(a))["phase_cycles"], dtype=float)
        # the same walker with its records staged in shared memory for the worm update
        eng.set_staging(192 * 1024)
        eng.sweep([a], n, measure=True)
        ms_staged, _ = eng.last_timing()
        c2 = np.array(eng.info(int(a))["phase_cycles"], dtype=float)
        eng.set_staging(0)
        line.update(cycles_per_sweep_diag_link_worm_measure=[round(x) for x in (c1 - c0) / n],
                    staged_cycles_per_sweep_diag_link_worm_measure=[round(x) for x in (c2 - c1) / n])
        t0 = time.perf_counter()
        eng.sweep([b], 500, measure=True, plain=True)
        plain_s = time.perf_counter() - t0
        eng.sweep([b], 500, measure=True, graph=True)
        graph_ms, _ = eng.last_timing()
        om = O.OracleModel(flat)
        w = O.OracleWalker(om, T=0.5, seed=args.seed, stream=0, thermalization=2000)
        w.init()
        w.run(2000, measure=False)
        t0 = time.perf_counter()
        w.run(n, measure=True)
        cpu_s = time.perf_counter() - t0
        line.update(config="8x8 S=1/2 Heisenberg, beta=2, one walker", gpu_persistent_sweeps_per_s=n / (ms / 1e3),
                    gpu_persistent_staged_sweeps_per_s=n / (ms_staged / 1e3),
                    gpu_plain_sweeps_per_s=500 / plain_s, gpu_graph_replay_sweeps_per_s=500 / (graph_ms / 1e3),
                    cpu_oracle_one_core_sweeps_per_s=n / cpu_s,
                    mean_L=eng.info(int(a))["L"])
        # the same model batched: 4096 walkers in one persistent launch, against the oracle with one
        # chain per host core (both after 2000 thermalisation sweeps)
        nb = 4096
        bids = eng.create_walkers(mid, [dict(T=0.5, seed=args.seed, stream=100 + k, thermalization=2000)
                                        for k in range(nb)])
        eng.init(bids)
        eng.sweep(bids, 2000, measure=False)
        eng.sweep(bids, 200, measure=True)
        bms = []
        for _ in range(3):
            eng.sweep(bids, 200, measure=True)
            bms.append(eng.last_timing()[0])
        nthreads = args.cpu_threads or os.cpu_count() or 1
        chains = [O.OracleWalker(om, T=0.5, seed=args.seed, stream=100 + k, thermalization=2000)
                  for k in range(nthreads)]
        for w in chains:
            w.init()
        O.run_parallel(om, chains, 2000, measure=False, nthreads=nthreads)
        t0 = time.perf_counter()
        O.run_parallel(om, chains, n, measure=True, nthreads=nthreads)
        cpu_all = nthreads * n / (time.perf_counter() - t0)
        line.update(batched_walkers=nb, gpu_batched_walker_sweeps_per_s=nb * 200 * 3 / (sum(bms) / 1e3),
                    cpu_oracle_all_cores_walker_sweeps_per_s=cpu_all, cpu_threads=nthreads)
    elif args.workload == "uneven":
        line.update(run_uneven_balanced(S, eng, args, rng))
    elif args.workload == "bilayer":
        line.update(run_bilayer(S, eng, args))
    elif args.workload == "serving":
        line.update(run_serving(args, 0, full=True))
    elif args.workload in ("magnet_bench", "cluster_bench"):
        line.update(run_reference_job(S, eng, args))
    eng.close()
    print(json.dumps(line), flush=True)


def balanced_counts(cost, kmax=4096):
    """Per-walker sweep counts for one cost-balanced block: walker i runs round(c_max / c_i) sweeps,
    c_i its device clock cycles per sweep in the last block, so that every walker works about as
    long as one sweep of the slowest."""
    cost = np.maximum(np.asarray(cost, dtype=np.float64), 1.0)
    return np.clip(np.rint(cost.max() / cost), 1, kmax).astype(np.int32)


class BalancedBlocks:
    """Cost-balanced sse_sweep_each blocks over a fixed set of walkers.  The counters of every walker
    (sweeps, device clock cycles, operator-updates = slot visits + worm steps) are read after each
    block; the next block gives walker i round(c_max / c_i) sweeps."""

    def __init__(self, eng, ids):
        self.eng, self.ids = eng, np.asarray(ids, dtype=np.int32)
        self.k = np.ones(len(self.ids), dtype=np.int32)
        self.cost = np.ones(len(self.ids))  # last measured clock cycles per sweep of every walker
        self.stopped = 0
        self.read()
        self.reset_totals()

    def reset_totals(self):
        """Start counting the sweeps and operator-updates of the following blocks, per walker id (a walker
        that stops keeps what it did in the blocks before)."""
        self.done_sw = {int(i): 0 for i in self.ids}
        self.done_ou = {int(i): 0.0 for i in self.ids}

    def _count(self, ids, sw0, ou0):
        pos = {int(i): j for j, i in enumerate(self.ids)}
        for i, a, b in zip(ids.tolist(), sw0.tolist(), ou0.tolist()):
            if i in pos:
                self.done_sw[i] += int(self.sw[pos[i]] - a)
                self.done_ou[i] += float(self.ou[pos[i]] - b)

    def read(self):
        inf = [self.eng.info(int(i)) for i in self.ids]
        self.info = inf
        self.sw = np.array([x["sweeps"] for x in inf], dtype=np.int64)
        self.cy = np.array([sum(x["phase_cycles"]) for x in inf], dtype=np.float64)
        self.ou = np.array([x["slot_visits"] + x["worm_steps"] for x in inf], dtype=np.float64)

    def block(self, measure=True, upto=None):
        """One block (at most `upto - sweeps` sweeps per walker when `upto` is given); returns its
        device seconds."""
        from sse_gb300.engine import SSEError

        k = self.k if upto is None else np.minimum(self.k, np.maximum(upto - self.sw, 0)).astype(np.int32)
        ids0, sw, cy, ou = self.ids, self.sw, self.cy, self.ou
        try:
            self.eng.sweep_each(self.ids, k, measure=measure)
        except SSEError:
            # a walker stopped (a measured worm past the step cap): the others finished the block;
            # the stopped ones leave the set
            ok = np.array([self.eng.info(int(i))["status"] == 0 for i in self.ids])
            self.stopped += int((~ok).sum())
            dev = self.eng.last_timing()[0] / 1e3
            self.ids, self.k, self.cost, sw, cy = self.ids[ok], self.k[ok], self.cost[ok], sw[ok], cy[ok]
            self.read()
            self._count(ids0[ok], sw, ou[ok])
            return dev
        dev = self.eng.last_timing()[0] / 1e3
        self.read()
        self._count(ids0, sw, ou)
        ran = self.sw - sw
        # walkers that ran no sweep in this block (done with thermalisation) keep their last cost
        self.cost = np.where(ran > 0, (self.cy - cy) / np.maximum(ran, 1), self.cost)
        self.k = balanced_counts(self.cost)
        return dev

    def thermalise(self, therm):
        """Blocks until every walker has done `therm` sweeps (the worm-count controller runs in all of
        them); returns (blocks, device seconds)."""
        blocks, dev = 0, 0.0
        while self.sw.min() < therm:
            dev += self.block(measure=True, upto=therm)
            blocks += 1
        return blocks, dev


def run_bilayer(S, eng, args):
    """The larger-local-space workload: S=1 Heisenberg antiferromagnet on a 48x48 periodic square
    bilayer (4608 sites, 11520 bonds), J=1, J_perp=0.5, Dz=0.3, hz=0.2, tables from the LP vertex
    builder; 2048 walkers, a third each at beta = 4, 8 and 16, in one batch.

    Opstring capacity is reserved up front at 1.25 x 13.2 N beta slots (the cutoff the reference's
    growth rule reaches; 13.2 N beta measured on the 12x12 bilayer), so that walkers do not stop for
    regrowth relaunches.  Thermalisation (`--therm` sweeps per walker, worm-count controller active)
    runs in cost-balanced sse_sweep_each blocks: every walker gets round(c_max / c_i) sweeps, capped
    at what it still needs, so a slow walker or a long early worm does not leave the batch idle for
    many sweeps.  Then `--steps` balanced blocks with measure! are timed."""
    p = {"lattice": {"unitcell": S.UnitCells.square_bilayer, "size": (48, 48)}, "S": 1.0, "J": 1.0, "Jp": 0.5,
         "parameter_map": {"J": ["Jp", "J", "J", "J", "J"]}, "Dz": 0.3, "hz": 0.2, "measure": ["magnetization"]}
    flat = S.flatten_model(S.MagnetModel(p))
    mid = eng.register_model(flat)
    betas = np.array([4.0, 8.0, 16.0])
    nw = 2048
    beta_of = betas[np.arange(nw) % 3]
    params = [dict(T=1.0 / float(beta_of[k]), seed=args.seed, stream=k, thermalization=args.therm) for k in range(nw)]
    ids = eng.create_walkers(mid, params)
    t0 = time.perf_counter()
    for b in betas:
        eng.reserve(ids[beta_of == b], int(1.25 * 13.2 * flat.nsites * b))
    eng.init(ids)

    bb = BalancedBlocks(eng, ids)
    blocks, therm_dev = bb.thermalise(args.therm)
    therm_s = time.perf_counter() - t0
    bb.reset_totals()
    dev = sum(bb.block(measure=True) for _ in range(args.steps))
    inf, k = bb.info, bb.k
    Ls = np.array([x["L"] for x in inf])
    live_beta = np.array([1.0 / x["T"] for x in inf])
    dsw = np.array([bb.done_sw[int(i)] for i in ids], dtype=np.float64)
    dou = np.array([bb.done_ou[int(i)] for i in ids], dtype=np.float64)
    # the CPU restatement on the same tables: 16 GPU walkers (every beta) exported and swept once on
    # the host cores, one chain per thread
    from oracle import oracle as O

    om = O.OracleModel(flat)
    nthreads = args.cpu_threads or os.cpu_count() or 1
    chains = []
    for j in range(min(nthreads, len(bb.ids))):
        wid = int(bb.ids[(j * len(bb.ids)) // min(nthreads, len(bb.ids))])
        ops, st, winf = eng.export(wid)
        w = O.OracleWalker(om, T=winf["T"], seed=args.seed, stream=0, thermalization=args.therm)
        w.set_opstring(ops, winf["num_operators"])
        w.set_state(st)
        w.w.ctr, w.w.num_worms, w.w.avg_worm_length, w.w.sweeps = (winf["rng_counter"], winf["num_worms"],
                                                                   winf["avg_worm_length"], winf["sweeps"])
        chains.append(w)
    t0 = time.perf_counter()
    O.run_parallel(om, chains, 1, measure=True, nthreads=nthreads)
    cpu_s = time.perf_counter() - t0
    cpu_ou = sum(w.w.worm_steps_total + w.w.slot_visits_total for w in chains)
    nops = np.array([x["num_operators"] for x in inf], dtype=np.float64)
    return dict(
        config="2048 walkers, S=1 square bilayer 48x48 (4608 sites), J=1, J_perp=0.5, Dz=0.3, hz=0.2, "
               "beta in {4,8,16} (a third each); cost-balanced sse_sweep_each blocks",
        thermalization_sweeps=args.therm, thermalization_blocks=blocks, thermalization_seconds_wall=therm_s,
        thermalization_seconds_device=therm_dev, steps=args.steps,
        walker_sweeps_per_s=float(dsw.sum()) / dev, operator_updates_per_s=float(dou.sum()) / dev,
        per_beta={str(b): {"walker_sweeps_per_s": float(dsw[beta_of == b].sum()) / dev,
                           "operator_updates_per_walker_sweep": float(dou[beta_of == b].sum() / max(dsw[beta_of == b].sum(), 1)),
                           "cutoff_L_median": int(np.median(Ls[live_beta == b])),
                           "operators_median": int(np.median(nops[live_beta == b]))} for b in betas.tolist()},
        regime=("the worm-count controller's transient: the reference's controller starts from an average worm "
                "length of 1 and adapts by 1% per sweep, so for many sweeps every sweep runs tens to hundreds of "
                "times the equilibrium 2n worm steps; operator-updates/s is the comparable rate"),
        cpu_baseline={"value": cpu_ou / cpu_s, "unit": "operator-updates/s", "cores": nthreads, "kind": "port",
                      "sample": f"{len(chains)} GPU walkers (all betas) exported and swept once on the host cores, "
                                "one chain per thread"},
        sweeps_per_block_min_median_max=[int(k.min()), int(np.median(k)), int(k.max())],
        walkers_stopped=bb.stopped,
        thermalisation_sweeps_undone_at_worm_cap=int(sum(x["worm_undos"] for x in inf)),
        cutoff_L_min_median_max=[int(Ls.min()), int(np.median(Ls)), int(Ls.max())])


def run_uneven_balanced(S, eng, args, rng):
    """The uneven batch / temperature sweep: 8192 walkers of S=1/2 Heisenberg square lattices, side
    in {8,16,24,32,48,64} and beta in {0.5,1,...,64} drawn uniformly from a seed (opstrings from about
    100 to 1.5 million slots).  Capacity is reserved up front from the projected cutoff.  The walkers
    thermalise for `--uneven-therm` sweeps each with the worm-count controller active, in
    cost-balanced sse_sweep_each blocks (walker i runs round(c_max / c_i) sweeps, c_i its device clock
    cycles per sweep in the previous block, capped at what it still needs); the autotuner
    (sse_autotune_each) then picks walkers per block and the shared-memory staging budget on such a
    block, and `--steps` balanced blocks with measure! are timed."""
    from sse_gb300.serving import projected_slots

    sides, betas = [8, 16, 24, 32, 48, 64], [0.5, 1, 2, 4, 8, 16, 32, 64]
    nw = 8192
    therm = args.uneven_therm
    pick = [(int(rng.choice(sides)), float(rng.choice(betas))) for _ in range(nw)]
    models = {L: eng.register_model(S.flatten_model(make_model(S, L))) for L in sides}
    ids = np.zeros(nw, dtype=np.int32)
    t0 = time.perf_counter()
    for L in sides:
        sel = [k for k, (l, _) in enumerate(pick) if l == L]
        got = eng.create_walkers(models[L], [dict(T=1.0 / pick[k][1], seed=args.seed, stream=k,
                                                  thermalization=therm) for k in sel])
        ids[sel] = got
        for b in betas:
            sub = np.array([got[j] for j, k in enumerate(sel) if pick[k][1] == b], dtype=np.int32)
            if len(sub):
                eng.reserve(sub, projected_slots(0.5, "square", L, b))
    eng.init(ids)
    bb = BalancedBlocks(eng, ids)
    blocks, therm_dev = bb.thermalise(therm)
    therm_s = time.perf_counter() - t0
    best_wpb, best_stage, probe_ms = eng.autotune_each(ids, bb.k, measure=True)
    bb.read()
    bb.reset_totals()
    dev = sum(bb.block(measure=True) for _ in range(args.steps))
    Ls = np.array([x["L"] for x in bb.info])
    ws = float(sum(bb.done_sw.values()))
    ou = float(sum(bb.done_ou.values()))
    k = bb.k
    return dict(config="8192 walkers, S=1/2 Heisenberg square L in {8..64}, beta in {0.5..64} uniform from a seed; "
                       "cost-balanced blocks (sse_sweep_each); thermalised with the worm-count controller active",
                thermalization_sweeps=therm, thermalization_blocks=blocks, thermalization_seconds_wall=therm_s,
                thermalization_seconds_device=therm_dev, steps=args.steps,
                walker_sweeps_per_s=ws / dev, operator_updates_per_s=ou / dev,
                sweeps_per_block_min_median_max=[int(k.min()), int(np.median(k)), int(k.max())],
                autotuned_warps_per_block=best_wpb, autotuned_stage_bytes=best_stage,
                walkers_stopped=bb.stopped,
                cutoff_L_min_median_max=[int(Ls.min()), int(np.median(Ls)), int(Ls.max())])


def reference_job_model(S, name):
    """The benchmark tasks of the reference's test/test_jobs.jl:113-167, timed there by
    test/benchmarks.jl:20-40 (one task: 2000 thermalisation + 5000 measured sweeps)."""
    if name == "magnet_bench":
        p = {"lattice": {"unitcell": S.UnitCells.square, "size": (10, 10)}, "J": 1.23, "hz": -0.2,
             "measure": S.all_magnetization_estimators(2)}
        return S.MagnetModel(p), 0.05, "10x10 square S=1/2, J=1.23, hz=-0.2, T=0.05, all magnetization estimators"
    p = {"inner_model": S.MagnetModel, "lattice": {"unitcell": S.UnitCells.fully_frust_square_bilayer, "size": (30, 30)},
         "parameter_map": {"S": ["Sa", "Sb"], "J": ["JD"] + ["JP"] * 8}, "cluster_bases": (S.ClusterBases.dimer,),
         "measure_quantum_numbers": [{"name": "", "quantum_number": 2}], "JD": 0.5, "JP": 1.0, "Sa": 0.5, "Sb": 0.5}
    return (S.ClusterModel(p), 0.1,
            "30x30 fully frustrated square bilayer in the dimer basis (900 dims-4 sites), JD=0.5, JP=1, T=0.1")


def run_reference_job(S, eng, args):
    """One of the reference's benchmark tasks: `--walkers` independent copies batched on the GPU, a single
    copy on the GPU, and the CPU oracle (one chain per core, and one chain on one core)."""
    from oracle import oracle as O

    model, T, desc = reference_job_model(S, args.workload)
    flat = S.flatten_model(model)
    mid = eng.register_model(flat)
    # the reference's task is 2000 + 5000 sweeps; --therm and --steps x --sweeps-per-step set the sample
    therm, sweeps = args.therm, args.steps * args.sweeps_per_step
    nw = args.walkers
    ids = eng.create_walkers(mid, [dict(T=T, seed=args.seed, stream=k, thermalization=therm) for k in range(nw)])
    eng.init(ids)
    t0 = time.perf_counter()
    ids, failed = sweep_tolerant(eng, ids, therm, measure=True)
    therm_dev = eng.last_timing()[0] / 1e3
    info0 = {i: eng.info(i) for i in ids.tolist()}
    ids, f = sweep_tolerant(eng, ids, sweeps, measure=True)
    failed += f
    meas_dev = eng.last_timing()[0] / 1e3
    wall = time.perf_counter() - t0
    info1 = {i: eng.info(i) for i in ids.tolist()}
    ou = sum(info1[i]["slot_visits"] + info1[i]["worm_steps"] - info0[i]["slot_visits"] - info0[i]["worm_steps"]
             for i in ids.tolist())
    # one copy alone on the GPU (latency-bound), a short sample
    (one,) = eng.create_walkers(mid, [dict(T=T, seed=args.seed, stream=nw + 1, thermalization=therm)])
    eng.init([one])
    n_single = max(1, min(200, sweeps // 10))
    eng.sweep([one], n_single, measure=True)
    eng.sweep([one], n_single, measure=True)
    single_s = eng.last_timing()[0] / 1e3
    # the CPU oracle: a bounded sample from a GPU-thermalised state
    om = O.OracleModel(flat)
    nthreads = args.cpu_threads or os.cpu_count() or 1
    chains = []
    for k, wid in enumerate(ids.tolist()[:nthreads]):
        ops, st, inf = eng.export(wid)
        w = O.OracleWalker(om, T=T, seed=args.seed, stream=k, thermalization=0)
        w.set_opstring(ops, inf["num_operators"])
        w.set_state(st)
        w.w.num_worms = inf["num_worms"]
        w.w.avg_worm_length = inf["avg_worm_length"]
        w.w.ctr = inf["rng_counter"]
        chains.append(w)
    cpu_sweeps = max(1, args.cpu_sweeps)
    t0 = time.perf_counter()
    chains[0].run(cpu_sweeps, measure=True)
    cpu_one = cpu_sweeps / (time.perf_counter() - t0)
    t0 = time.perf_counter()
    O.run_parallel(om, chains, cpu_sweeps, measure=True, nthreads=nthreads)
    cpu_all = len(chains) * cpu_sweeps / (time.perf_counter() - t0)
    Ls = np.array([info1[i]["L"] for i in ids.tolist()])
    return dict(
        config=desc, reference_task="2000 thermalisation + 5000 measured sweeps per walker",
        thermalization_sweeps=therm, measured_sweeps=sweeps, cpu_sample_sweeps=cpu_sweeps,
        walkers=nw, walkers_stopped_by_worm_cap=failed,
        thermalisation_sweeps_undone_at_worm_cap=sum(info1[i]["worm_undos"] for i in ids.tolist()),
        gpu_batched_walker_sweeps_per_s=len(ids) * sweeps / meas_dev,
        gpu_batched_operator_updates_per_s=ou / meas_dev,
        gpu_batched_job_seconds_device=therm_dev + meas_dev, gpu_batched_job_seconds_wall=wall,
        gpu_single_walker_sweeps_per_s=n_single / single_s,
        cpu_oracle_one_core_sweeps_per_s=cpu_one,
        cpu_oracle_all_cores_walker_sweeps_per_s=cpu_all, cpu_threads=nthreads,
        cutoff_L_min_median_max=[int(Ls.min()), int(np.median(Ls)), int(Ls.max())],
    )


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload != "uniform":
        run_other_workload(args)
        return
    rank, world, local = dist_setup(args)
    S = _sse_loader.load()
    from sse_gb300.engine import Engine

    flat = S.flatten_model(make_model(S, args.side))
    N = flat.nsites
    eng = Engine(local)
    mid = eng.register_model(flat)
    nw = args.walkers
    ids = eng.create_walkers(mid, [dict(T=1.0 / args.beta, seed=args.seed, stream=st, thermalization=args.therm)
                                   for st in replica_streams(rank, nw)])
    eng.init(ids)
    # thermalisation (controller active), in blocks
    done = 0
    while done < args.therm:
        blk = min(100, args.therm - done)
        eng.sweep(ids, blk, measure=True)
        done += blk
    # walkers per block and the shared-memory staging budget from the autotuner (its probes are
    # real Carlo steps of the thermalised batch)
    if args.wpb:
        eng.set_launch(args.wpb, 0)
        tuned_wpb, tuned_stage = args.wpb, 0
    else:
        tuned_wpb, tuned_stage, _ = eng.autotune(ids, nsweeps_probe=5, measure=True)
    # the sweep blocks run as CUDA-graph replays (the first warm-up step captures the block)
    for _ in range(args.warmup):
        eng.sweep(ids, args.sweeps_per_step, measure=True, graph=True)
        eng.observables(ids, reset=True)

    info0 = [eng.info(int(i)) for i in ids]
    clocks = ClockSampler(local)
    barrier(world)
    clocks.start()
    step_ms = []
    launches = 0
    if args.profile:
        eng.profiler_range(True)
    for _ in range(args.steps):
        eng.sweep(ids, args.sweeps_per_step, measure=True, graph=True)
        ms, nl = eng.last_timing()
        step_ms.append(ms)
        launches += nl
    if args.profile:
        eng.profiler_range(False)
    clk = clocks.stop()
    barrier(world)
    info1 = [eng.info(int(i)) for i in ids]
    dev_s = sum(step_ms) / 1e3
    t_max = barrier_max(world, dev_s)
    total_ws = barrier_sum(world, nw * args.sweeps_per_step * args.steps)
    value = total_ws / t_max

    slots = sum(b["slot_visits"] - a["slot_visits"] for a, b in zip(info0, info1))
    worm = sum(b["worm_steps"] - a["worm_steps"] for a, b in zip(info0, info1))
    opupd = barrier_sum(world, slots + worm) / t_max
    # algorithmic bytes per launch of the sweep kernel (one launch per step)
    nsw = args.sweeps_per_step * args.steps
    bytes_total = sum(walker_bytes((b["slot_visits"] - a["slot_visits"]) / nsw, (b["worm_steps"] - a["worm_steps"]) / nsw, N) * nsw
                      for a, b in zip(info0, info1))
    per_launch_bytes = bytes_total / args.steps
    avg_launch_s = dev_s / args.steps
    achieved = per_launch_bytes / avg_launch_s / 1e9
    peak, peak_kind = load_peaks()
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "k_walk_sweep_traffic.json")
    if os.path.exists(tfile):
        try:
            with open(tfile) as f:
                tj = json.load(f)
            traffic = float(tj["dram_bytes_per_walker_sweep"]) * nw * args.sweeps_per_step
        except Exception:
            traffic = None

    # end-to-end through the public API: ids H2D, sweep, observables D2H, wall clock
    barrier(world)
    t0 = time.perf_counter()
    obs_bytes = 0
    for _ in range(args.steps):
        eng.sweep(ids, args.sweeps_per_step, measure=True, graph=True)
        out = eng.observables(ids, reset=True)
        obs_bytes = sum(s.nbytes + c.nbytes + l.nbytes for s, c, l in out)
    e2e_s = barrier_max(world, time.perf_counter() - t0)
    e2e_value = total_ws / e2e_s

    # the same sweep block launched directly instead of from the captured graph
    direct_ms = []
    for _ in range(min(2, args.steps)):
        eng.sweep(ids, args.sweeps_per_step, measure=True)
        direct_ms.append(eng.last_timing()[0])
    direct_value = nw * args.sweeps_per_step / (np.mean(direct_ms) / 1e3) if direct_ms else None

    result = None
    if rank == 0:
        nchk = min(16, nw, args.cpu_threads or os.cpu_count() or 1)
        states = [eng.export(int(i)) for i in ids[: max(nchk, args.cpu_threads or os.cpu_count() or 1)]]
        parity = parity_check(S, flat, eng, ids, states[:nchk], args)
        # plain path: one launch per walker per sweep (a per-walker sweep! call)
        sub = ids[: args.plain_walkers]
        eng.sweep(sub, 1, measure=True, plain=True)
        t0 = time.perf_counter()
        eng.sweep(sub, 2, measure=True, plain=True)
        plain_s = time.perf_counter() - t0
        plain_value = len(sub) * 2 / plain_s

        cpu = cpu_baseline(S, flat, states, args, args.cpu_threads or os.cpu_count() or 1)
        serving = run_serving(args, local) if args.serving_requests > 0 else None

        mean_L = float(np.mean([x["L"] for x in info1]))
        cyc = np.array([np.array(b["phase_cycles"], dtype=float) - np.array(a["phase_cycles"], dtype=float)
                        for a, b in zip(info0, info1)])
        work = np.array([(b["worm_steps"] - a["worm_steps"]) + (b["slot_visits"] - a["slot_visits"])
                         for a, b in zip(info0, info1)], dtype=float)
        phases = dict(zip(["diagonal", "link", "worm", "measure"], (cyc.sum(0) / cyc.sum()).round(4).tolist()))
        worm_steps = sum(b["worm_steps"] - a["worm_steps"] for a, b in zip(info0, info1))
        slots = sum(b["slot_visits"] - a["slot_visits"] for a, b in zip(info0, info1))
        # what bounds the kernel: one dependent DRAM access per worm step, one warp per walker
        latency = {"worm_cycles_per_step": float(cyc[:, 2].sum() / max(worm_steps, 1)),
                   "diag_cycles_per_slot": float(cyc[:, 0].sum() / max(slots, 1)),
                   "link_cycles_per_slot": float(cyc[:, 1].sum() / max(slots, 1)),
                   "dram_pointer_chase_cycles": 790,
                   "note": "per-walker SM clock cycles under full load; a lone dependent DRAM access costs about "
                           "790 cycles on this GPU"}
        result = {
            "metric": METRIC,
            "value": value,
            "unit": METRIC,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": t_max * 1e3 / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "i32+f64",
            "data": "synthetic",
            "config": {
                "workload": workload_name(args),
                "walkers": nw,
                "side": args.side,
                "beta": args.beta,
                "thermalization_sweeps": args.therm,
                "sweeps_per_step": args.sweeps_per_step,
                "parallelism": f"replicas x{world}",
                "l2": f"working set {sum(x['capacity'] for x in info1) * 40 / 1e9:.1f} GB of walker state, larger than L2",
                "mean_cutoff_L": mean_L,
                "autotuned_walkers_per_block": tuned_wpb,
                "autotuned_stage_bytes": tuned_stage,
            },
            "operator_updates_per_s": opupd,
            "phase_cycle_share": phases,
            "latency": latency,
            "load_balance_mean_over_max_walker_work": float(work.mean() / work.max()),
            "plain": {"value": plain_value, "unit": METRIC, "walkers": len(sub),
                      "path": "one kernel launch (one warp) per walker per sweep, synchronised after each"},
            "batched_over_plain": value / plain_value,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_kind": peak_kind, "kernel": "k_walk<SWEEP>",
                         "algorithmic_bytes_per_launch": per_launch_bytes},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": 4 * len(ids),
                    "d2h_bytes_per_step": obs_bytes},
            "gpu_launches": launches,
            "launch_path": "CUDA-graph replay of the sweep block (flag/queue resets + one persistent launch)",
            "direct_launch_value": direct_value,
            "parity_checked": not parity["mismatched_walkers"],
            "parity": parity,
            "clocks": clk,
            "serving": serving,
        }
        print(json.dumps(result), flush=True)
    eng.close()
    if result is not None and not result["parity_checked"]:
        sys.exit("bench: the benchmarked walkers left the oracle's chain: " + str(result["parity"]))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
