"""GPU chains in the benchmarked regime, continued side by side with the oracle.

The short-horizon parity tests start both sides at Carlo.init! and compare after a few dozen
sweeps, while the cutoff is still on its growth ladder.  These tests thermalise walkers on the GPU
for hundreds of sweeps first -- long opstrings, a settled worm-count controller, the diagonal
update's rare ambiguous-lane and FP64 fallback paths live -- then export them through the C ABI,
import each into an oracle walker and run both for more sweeps.  Everything must stay equal bit for
bit: opstring, spin state, cutoff, operator count, replay counter, the controller's doubles and the
worm-step counts; the observables accumulated over the continuation to 1e-12 relative.

* 32x32 S=1/2 Heisenberg at beta = 16 (the benchmark workload): 500 sweeps on the GPU, then 20
  more on both sides that cross the end of thermalisation (10 with the controller active, 10
  measured).
* 16x16 at beta = 8: 1000 sweeps, then 50 measured sweeps, for more walkers.
* the S=1 square bilayer with anisotropy and field (the larger-local-space workload's model) at
  12x12, beta = 8, from Carlo.init! with the worm-step cap lowered to its minimum for the first
  sweeps, so that long thermalisation worms are undone, and continued after export.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def square(S, side):
    return S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (side, side)},
                                          "J": 1.0, "measure": ["magnetization", "staggered_magnetization"]}))


def bilayer_s1(S, side):
    return S.flatten_model(S.MagnetModel({
        "lattice": {"unitcell": S.UnitCells.square_bilayer, "size": (side, side)}, "S": 1.0, "J": 1.0, "Jp": 0.5,
        "parameter_map": {"J": ["Jp", "J", "J", "J", "J"]}, "Dz": 0.3, "hz": 0.2, "measure": ["magnetization"]}))


def oracle_from_export(O, om, ops, st, inf, p):
    """An oracle walker holding the exported GPU walker's chain (the checkpoint fields)."""
    w = O.OracleWalker(om, T=p["T"], seed=p["seed"], stream=p["stream"], thermalization=p["thermalization"])
    w.set_opstring(ops, inf["num_operators"])
    w.set_state(st)
    w.w.ctr = inf["rng_counter"]
    w.w.num_worms = inf["num_worms"]
    w.w.avg_worm_length = inf["avg_worm_length"]
    w.w.sweeps = inf["sweeps"]
    return w


def continue_and_compare(O, eng, flat, ids, params, nsweeps, cap_factor=0):
    """Export `ids`, continue them `nsweeps` sweeps on the GPU and in the oracle, compare."""
    om = O.OracleModel(flat)
    chains, steps0 = [], []
    for wid, p in zip(ids.tolist(), params):
        ops, st, inf = eng.export(wid)
        assert inf["status"] == 0
        w = oracle_from_export(O, om, ops, st, inf, p)
        if cap_factor:
            w.w.worm_cap_factor = cap_factor
        chains.append(w)
        steps0.append(inf["worm_steps"])
    eng.observables(ids, reset=True)
    eng.sweep(ids, nsweeps, measure=True)
    O.run_parallel(om, chains, nsweeps, measure=True, nthreads=min(16, len(chains)))
    for wid, w, s0 in zip(ids.tolist(), chains, steps0):
        ops, st, inf = eng.export(wid)
        assert inf["status"] == w.w.status == 0
        assert inf["L"] == w.w.L and inf["num_operators"] == w.w.num_operators and inf["sweeps"] == w.w.sweeps
        assert inf["rng_counter"] == w.w.ctr
        assert inf["num_worms"] == w.w.num_worms and inf["avg_worm_length"] == w.w.avg_worm_length
        assert inf["worm_steps"] - s0 == w.w.worm_steps_total
        assert np.array_equal(ops, w.ops) and np.array_equal(st, w.state)
        s, c, _ = eng.observables([wid])[0]
        so, co, _ = w.obs()
        assert np.array_equal(c, co)
        np.testing.assert_allclose(s, so, rtol=RTOL, atol=0)
    return chains


def test_headline_walkers_after_500_sweeps_continue_like_oracle(S, O):
    from sse_gb300.engine import Engine

    flat = square(S, 32)
    eng = Engine(0)
    try:
        mid = eng.register_model(flat)
        params = [dict(T=1.0 / 16, seed=9001, stream=k, thermalization=510) for k in range(4)]
        ids = eng.create_walkers(mid, params)
        eng.init(ids)
        for _ in range(5):
            eng.sweep(ids, 100, measure=True)
        infos = [eng.info(int(i)) for i in ids]
        assert all(x["sweeps"] == 500 and x["L"] > 45_000 for x in infos)
        chains = continue_and_compare(O, eng, flat, ids, params, 20)
        # the continuation crossed the end of thermalisation: 10 measured sweeps each
        assert all(int(w.obs()[1][0]) == 10 for w in chains)
    finally:
        eng.close()


def test_batch_after_1000_sweeps_continues_like_oracle(S, O):
    from sse_gb300.engine import Engine

    flat = square(S, 16)
    eng = Engine(0)
    try:
        mid = eng.register_model(flat)
        params = [dict(T=1.0 / 8, seed=9002, stream=k, thermalization=600) for k in range(64)]
        ids = eng.create_walkers(mid, params)
        eng.init(ids)
        for _ in range(10):
            eng.sweep(ids, 100, measure=True)
        pick = np.arange(0, 64, 8)
        continue_and_compare(O, eng, flat, ids[pick], [params[k] for k in pick.tolist()], 50)
    finally:
        eng.close()


def test_s1_bilayer_with_undone_worms_matches_oracle(S, O):
    """12x12 S=1 bilayer (J=1, J_perp=0.5, Dz=0.3, hz=0.2) at beta = 8: 16 chains from Carlo.init!,
    the first 10 sweeps with the worm-step cap at its minimum (factor 1: max(L + 16, 2^16) steps), so
    that long early worms undo their sweep's worm phase, then 50 sweeps under the default cap, of
    which 30 are measured.  Equal to the oracle's chains, with the same undo counts; then 50 more
    sweeps after export."""
    from sse_gb300.engine import Engine

    flat = bilayer_s1(S, 12)
    eng = Engine(0)
    try:
        mid = eng.register_model(flat)
        params = [dict(T=1.0 / 8, seed=9003, stream=k, thermalization=30) for k in range(16)]
        ids = eng.create_walkers(mid, params)
        eng.set_worm_cap(ids, 1)
        eng.init(ids)
        eng.sweep(ids, 10, measure=True)
        eng.set_worm_cap(ids, 64)
        eng.sweep(ids, 50, measure=True)
        om = O.OracleModel(flat)
        chains = []
        for p in params:
            w = O.OracleWalker(om, T=p["T"], seed=p["seed"], stream=p["stream"], thermalization=p["thermalization"])
            w.w.worm_cap_factor = 1
            w.init()
            chains.append(w)
        O.run_parallel(om, chains, 10, measure=True, nthreads=16)
        for w in chains:
            w.w.worm_cap_factor = 64
        O.run_parallel(om, chains, 50, measure=True, nthreads=16)
        undos = 0
        for wid, w in zip(ids.tolist(), chains):
            ops, st, inf = eng.export(wid)
            assert inf["status"] == w.w.status == 0
            assert inf["L"] == w.w.L and inf["rng_counter"] == w.w.ctr
            assert inf["num_worms"] == w.w.num_worms and inf["avg_worm_length"] == w.w.avg_worm_length
            assert inf["worm_undos"] == w.w.worm_undos
            assert np.array_equal(ops, w.ops) and np.array_equal(st, w.state)
            s, c, _ = eng.observables([wid])[0]
            so, co, _ = w.obs()
            assert np.array_equal(c, co)
            np.testing.assert_allclose(s, so, rtol=RTOL, atol=0)
            undos += inf["worm_undos"]
        assert undos >= 1, "no thermalisation worm phase was undone; lower cap did not bite"
        continue_and_compare(O, eng, flat, ids, params, 50)
    finally:
        eng.close()
