"""GPU engine vs the CPU oracle, through the C ABI.

Integer state (opstring, spin state, operator count, cutoff, replay counter)
and the worm controller's FP64 scalars must match bit for bit.  FP64
estimators must match within 1e-12 relative (the engine sums the running
magnetisation with a warp scan instead of the reference's sequential loop).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module")
def eng():
    from sse_gb300.engine import Engine

    e = Engine(0)
    yield e
    e.close()


def sq_model(S, L=8, measure=("magnetization", "staggered_magnetization")):
    return S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (L, L)}, "J": 1.0, "measure": list(measure)})


def honeycomb_mixed(S):
    return S.MagnetModel({"lattice": {"unitcell": S.UnitCells.honeycomb, "size": (4, 4)}, "J": 1.4,
                          "parameter_map": {"S": ("S1", "S2")}, "S1": 0.5, "S2": 1.0,
                          "measure": S.all_magnetization_estimators(2)})


def bilayer_s1(S, L=4):
    return S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square_bilayer, "size": (L, L)}, "S": 1.0, "J": 1.0,
                          "Jp": 0.5, "parameter_map": {"J": ["Jp", "J", "J", "J", "J"]}, "Dz": 0.3, "hz": 0.2,
                          "measure": ["magnetization"]})


def cluster_dimer(S):
    """The reference's cluster ED job (test/test_jobs.jl:69-110): dims-4 dimer sites, signed tables."""
    return S.ClusterModel({
        "inner_model": S.MagnetModel,
        "lattice": {"unitcell": S.UnitCells.fully_frust_square_bilayer, "size": (3, 2)},
        "parameter_map": {"S": ["Sa", "Sb"], "J": ["JD", "JxP", "JxP", "JyP", "JyP", "JxX", "JxX", "JyX", "JyX"]},
        "cluster_bases": (S.ClusterBases.dimer,),
        "measure_quantum_numbers": [{"name": "", "quantum_number": 2}],
        "JD": 1, "JxP": 0.55, "JyP": 0.6, "JxX": 0.7, "JyX": 0.3, "d": -0.2, "Dz": 0.2, "Dx": 0.5,
        "Sa": 0.5, "Sb": 0.5})


_FLAT = {}


def flat_of(S, name):
    if name not in _FLAT:
        m = {"sq8": lambda: sq_model(S), "honey": lambda: honeycomb_mixed(S), "bilayer": lambda: bilayer_s1(S),
             "sq32": lambda: sq_model(S, 32), "sq4": lambda: sq_model(S, 4),
             "cluster": lambda: cluster_dimer(S)}[name]()
        _FLAT[name] = S.flatten_model(m)
    return _FLAT[name]


def compare(eng, O, flat, wid, w, obs=True):
    ops, st, inf = eng.export(wid)
    assert inf["status"] == 0
    assert inf["L"] == w.w.L
    assert inf["num_operators"] == w.w.num_operators
    assert inf["rng_counter"] == w.w.ctr
    assert np.array_equal(ops, w.ops)
    assert np.array_equal(st, w.state)
    assert inf["num_worms"] == w.w.num_worms
    assert inf["avg_worm_length"] == w.w.avg_worm_length
    assert inf["sweeps"] == w.w.sweeps
    assert inf["worm_steps"] == w.w.worm_steps_total
    if obs:
        s, c, last = eng.observables([wid])[0]
        so, co, lo = w.obs()
        assert np.array_equal(c, co)
        np.testing.assert_allclose(s, so, rtol=RTOL, atol=0)
        np.testing.assert_allclose(last, lo, rtol=RTOL, atol=0)


def test_gpu_vertex_list_golden(S, eng):
    from test_oracle import golden_expected, golden_model, golden_ops

    flat = golden_model(S)
    mid = eng.register_model(flat)
    (wid,) = eng.create_walkers(mid, [dict(T=1.0, seed=1, stream=0)])
    ops = golden_ops()
    eng.import_(wid, ops, np.zeros(4, np.uint8), dict(num_operators=int(np.count_nonzero(ops))))
    v, vf, vl = eng.vertex_list(wid)
    exp, evf, evl = golden_expected()
    assert np.array_equal(v, exp)
    assert np.array_equal(vf, evf)
    assert np.array_equal(vl, evl)


@pytest.mark.parametrize("name,T", [("sq8", 0.5), ("honey", 0.1), ("bilayer", 0.25), ("sq4", 4.0), ("cluster", 0.3),
                                    ("cluster", 0.05)])
def test_gpu_init_and_sweeps_match_oracle(S, O, eng, name, T):
    flat = flat_of(S, name)
    mid = eng.register_model(flat)
    params = [dict(T=T, seed=99, stream=k, thermalization=12) for k in range(3)]
    ids = eng.create_walkers(mid, params)
    eng.init(ids)
    om = O.OracleModel(flat)
    ws = []
    for k, wid in enumerate(ids.tolist()):
        w = O.OracleWalker(om, T=T, seed=99, stream=k, thermalization=12)
        w.init()
        compare(eng, O, flat, wid, w, obs=False)
        ws.append(w)
    # thermalisation (controller active) then measured sweeps, in two calls
    eng.sweep(ids, 10, measure=True)
    eng.sweep(ids, 15, measure=True)
    for wid, w in zip(ids.tolist(), ws):
        w.run(25, measure=True)
        compare(eng, O, flat, wid, w)


def test_gpu_plain_path_equals_batched(S, O, eng):
    flat = flat_of(S, "sq8")
    mid = eng.register_model(flat)
    a = eng.create_walkers(mid, [dict(T=0.5, seed=7, stream=k, thermalization=2) for k in range(3)])
    b = eng.create_walkers(mid, [dict(T=0.5, seed=7, stream=k, thermalization=2) for k in range(3)])
    eng.init(a)
    eng.init(b)
    eng.sweep(a, 8, measure=True)
    eng.sweep(b, 8, measure=True, plain=True)
    for x, y in zip(a.tolist(), b.tolist()):
        oa, sa, ia = eng.export(x)
        ob, sb, ib = eng.export(y)
        assert np.array_equal(oa, ob) and np.array_equal(sa, sb)
        assert ia["rng_counter"] == ib["rng_counter"] and ia["num_worms"] == ib["num_worms"]


def test_gpu_result_independent_of_batch(S, O, eng):
    """A walker's trajectory depends only on its own (seed, stream): alone or mixed
    with other models and temperatures it ends in the same state."""
    f8, fh, fb = flat_of(S, "sq8"), flat_of(S, "honey"), flat_of(S, "bilayer")
    m8, mh, mb = eng.register_model(f8), eng.register_model(fh), eng.register_model(fb)
    alone = eng.create_walkers(m8, [dict(T=0.3, seed=5, stream=11, thermalization=3)])
    mixed = [eng.create_walkers(m8, [dict(T=0.3, seed=5, stream=11, thermalization=3)])[0]]
    mixed += eng.create_walkers(mh, [dict(T=0.2, seed=6, stream=k) for k in range(4)]).tolist()
    mixed += eng.create_walkers(mb, [dict(T=1.0, seed=8, stream=k) for k in range(4)]).tolist()
    eng.init(alone)
    eng.init(mixed)
    eng.sweep(alone, 12)
    eng.sweep(mixed, 12)
    oa, sa, ia = eng.export(int(alone[0]))
    om, sm, im = eng.export(mixed[0])
    assert np.array_equal(oa, om) and np.array_equal(sa, sm) and ia["rng_counter"] == im["rng_counter"]
    np.testing.assert_array_equal(eng.observables([int(alone[0])])[0][0], eng.observables([mixed[0]])[0][0])


def test_gpu_regrowth_from_tiny_capacity(S, O, eng):
    """Cutoff growth (src/sse.jl:138-145) beyond the reserved capacity relaunches without changing the chain."""
    flat = flat_of(S, "sq8")
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=0.05, seed=3, stream=k, init_opstring_cutoff=0) for k in range(2)])
    eng.init(ids)
    eng.sweep(ids, 20, measure=False)
    om = O.OracleModel(flat)
    for k, wid in enumerate(ids.tolist()):
        w = O.OracleWalker(om, T=0.05, seed=3, stream=k)
        w.init(init_cutoff=0)
        w.run(20, measure=False)
        compare(eng, O, flat, wid, w, obs=False)
        assert eng.info(wid)["capacity"] >= w.w.L


def test_gpu_export_import_roundtrip(S, O, eng):
    flat = flat_of(S, "honey")
    mid = eng.register_model(flat)
    a, b = eng.create_walkers(mid, [dict(T=0.2, seed=4, stream=1, thermalization=5), dict(T=0.2, seed=4, stream=1, thermalization=5)])
    eng.init([a])
    eng.sweep([a], 7)
    ops, st, inf = eng.export(int(a))
    eng.import_(int(b), ops, st, inf)
    eng.sweep([a], 9)
    eng.sweep([b], 9)
    oa, sa, ia = eng.export(int(a))
    ob, sb, ib = eng.export(int(b))
    assert np.array_equal(oa, ob) and np.array_equal(sa, sb) and ia["rng_counter"] == ib["rng_counter"]


def test_gpu_empty_opstrings_high_temperature(S, O, eng):
    """Very high T: the opstring is often empty (n = 0), worms are skipped and every
    site is redrawn (src/sse.jl:221-222, 234-236)."""
    flat = flat_of(S, "sq4")
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=50.0, seed=21, stream=k, init_opstring_cutoff=0, thermalization=4) for k in range(4)])
    eng.init(ids)
    eng.sweep(ids, 30, measure=True)
    om = O.OracleModel(flat)
    for k, wid in enumerate(ids.tolist()):
        w = O.OracleWalker(om, T=50.0, seed=21, stream=k, thermalization=4)
        w.init(init_cutoff=0)
        w.run(30, measure=True)
        compare(eng, O, flat, wid, w)


def test_gpu_32x32_beta16_matches_oracle(S, O, eng):
    """The benchmark workload's model at its temperature, a few full sweeps from a fresh start."""
    flat = flat_of(S, "sq32")
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=1 / 16, seed=2026, stream=k, thermalization=100) for k in range(2)])
    eng.init(ids)
    eng.sweep(ids, 12, measure=True)
    om = O.OracleModel(flat)
    for k, wid in enumerate(ids.tolist()):
        w = O.OracleWalker(om, T=1 / 16, seed=2026, stream=k, thermalization=100)
        w.init()
        w.run(12, measure=True)
        compare(eng, O, flat, wid, w)


def test_gpu_graph_replay_equals_launch(S, O, eng):
    """Sweep blocks replayed from a captured CUDA graph give the same chains as direct launches,
    including blocks where walkers regrow (relaunches outside the graph)."""
    flat = flat_of(S, "sq8")
    mid = eng.register_model(flat)
    a = eng.create_walkers(mid, [dict(T=0.2, seed=12, stream=k, init_opstring_cutoff=0, thermalization=3) for k in range(5)])
    b = eng.create_walkers(mid, [dict(T=0.2, seed=12, stream=k, init_opstring_cutoff=0, thermalization=3) for k in range(5)])
    eng.init(a)
    eng.init(b)
    for _ in range(4):  # capture on the first block, replay on the others
        eng.sweep(a, 6, measure=True, graph=True)
        eng.sweep(b, 6, measure=True)
    for x, y in zip(a.tolist(), b.tolist()):
        oa, sa, ia = eng.export(x)
        ob, sb, ib = eng.export(y)
        assert np.array_equal(oa, ob) and np.array_equal(sa, sb) and ia["rng_counter"] == ib["rng_counter"]
        np.testing.assert_array_equal(eng.observables([x])[0][0], eng.observables([y])[0][0])


def test_gpu_autotune_keeps_parity(S, O, eng):
    flat = flat_of(S, "honey")
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=0.3, seed=8, stream=k, thermalization=50) for k in range(6)])
    eng.init(ids)
    best, stage, ms = eng.autotune(ids, nsweeps_probe=3, measure=True)
    assert best in (1, 2, 4) and stage >= 0 and ms > 0
    eng.sweep(ids, 4, measure=True)
    eng.set_launch(0, 0)
    eng.set_staging(0)
    om = O.OracleModel(flat)
    for k, wid in enumerate(ids.tolist()):
        done = eng.info(wid)["sweeps"]  # probe sweeps (3 per candidate) + 4
        assert done >= 3 * 3 + 4 and (done - 4) % 3 == 0
        w = O.OracleWalker(om, T=0.3, seed=8, stream=k, thermalization=50)
        w.init()
        w.run(done, measure=True)
        compare(eng, O, flat, wid, w)


@pytest.mark.parametrize("name,T,stage", [("sq8", 0.5, 4096), ("sq8", 0.5, 192 * 1024), ("honey", 0.1, 16384),
                                          ("bilayer", 0.25, 32768), ("cluster", 0.3, 65536), ("sq4", 4.0, 2048)])
def test_gpu_shared_memory_staging_matches_oracle(S, O, eng, name, T, stage):
    """Walkers whose records fit the staging budget run the worm update in shared memory; the rest
    (and the same walker in sweeps where its operator count exceeds the budget) chase through HBM.
    Either way the chain is the oracle's, bit for bit, including cutoff growth from a tiny start."""
    flat = flat_of(S, name)
    mid = eng.register_model(flat)
    params = [dict(T=T, seed=17, stream=k, thermalization=6, init_opstring_cutoff=0 if k == 0 else -1)
              for k in range(4)]
    ids = eng.create_walkers(mid, params)
    eng.init(ids)
    eng.set_staging(stage)
    try:
        eng.sweep(ids, 9, measure=True)
        eng.sweep(ids, 7, measure=True, plain=True)
        eng.sweep(ids, 5, measure=True, graph=True)
    finally:
        eng.set_staging(0)
    om = O.OracleModel(flat)
    for p, wid in zip(params, ids.tolist()):
        w = O.OracleWalker(om, T=T, seed=17, stream=p["stream"], thermalization=6)
        w.init(init_cutoff=p["init_opstring_cutoff"])
        w.run(21, measure=True)
        compare(eng, O, flat, wid, w)


def test_gpu_staging_argument_checks(eng):
    from sse_gb300.engine import SSEError

    with pytest.raises(SSEError):
        eng.set_staging(-1)
    with pytest.raises(SSEError):
        eng.set_staging(10**7)
    eng.set_staging(1000)
    assert eng.get_staging() == 1024  # rounded to 32 bytes
    eng.set_staging(0)
    assert eng.get_staging() == 0


def test_gpu_autotune_each_keeps_parity(S, O, eng):
    """Probing launch shapes and staging budgets with per-walker sweep counts runs real Carlo steps:
    every walker ends exactly where the oracle does after the same number of steps."""
    flat = flat_of(S, "sq4")
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=0.4, seed=31, stream=k, thermalization=5) for k in range(5)])
    eng.init(ids)
    ns = np.array([1, 3, 2, 1, 4], dtype=np.int32)
    best, stage, ms = eng.autotune_each(ids, ns, measure=True)
    assert best in (1, 2, 4) and stage >= 0 and ms > 0
    eng.set_launch(0, 0)
    eng.set_staging(0)
    om = O.OracleModel(flat)
    nprobe = eng.info(int(ids[0]))["sweeps"] // int(ns[0])
    for k, wid in enumerate(ids.tolist()):
        assert eng.info(wid)["sweeps"] == nprobe * int(ns[k])
        w = O.OracleWalker(om, T=0.4, seed=31, stream=k, thermalization=5)
        w.init()
        w.run(nprobe * int(ns[k]), measure=True)
        compare(eng, O, flat, wid, w)
