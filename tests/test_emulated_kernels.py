"""The engine's own kernels, run on the CPU on emulated warps (tests/warp_emu), against the oracle.

The emulated library is built from the engine's device sources with two textual substitutions
(the PTX lane-mask read and the dynamic shared-memory declaration; see tests/warp_emu/build.py).  It
runs every launch of the C ABI's host code, with the fake CUDA runtime of tests/fake_cuda as device
memory.  So these tests check the kernels' logic, bit for bit against the oracle, without a GPU:
the diagonal update, linking, worms, the controller, measurement, cutoff growth, staging, the plain
and cost-balanced paths, tempering, the invariant check and the worm cap.  What they cannot check
is what only the hardware does: the compiled sm_103a code, memory ordering between warps, timing.
The GPU tests (-m gpu) check those, with the same oracle.
"""

import numpy as np
import pytest

from golden_cases import CASES


@pytest.fixture
def eng(emu):
    from sse_gb300.engine import Engine

    e = Engine(0, library=emu)
    yield e
    e.close()


def compare(eng, flat, wid, w, measured=True, counters=True):
    """Engine walker `wid` against oracle walker `w`: everything bit for bit (`counters`: also the
    cumulative worm-step count, a diagnostic that an imported walker starts afresh)."""
    ops, st, inf = eng.export(int(wid))
    assert inf["status"] == w.w.status
    assert inf["L"] == w.w.L and inf["num_operators"] == w.w.num_operators and inf["sweeps"] == w.w.sweeps
    assert inf["rng_counter"] == w.w.ctr
    assert inf["num_worms"] == w.w.num_worms and inf["avg_worm_length"] == w.w.avg_worm_length
    if counters:
        assert inf["worm_steps"] == w.w.worm_steps_total
    assert np.array_equal(ops, w.ops) and np.array_equal(st, w.state)
    if measured:
        s, c, _ = eng.observables([int(wid)])[0]
        so, co, _ = w.obs()
        assert np.array_equal(c, co)
        np.testing.assert_array_equal(s, so)


@pytest.mark.parametrize("case", list(CASES)[:4])
def test_emulated_sweeps_match_oracle(S, O, eng, case):
    """The golden cases' model families (S=1/2 square, mixed-spin honeycomb, S=1 bilayer with field
    and anisotropy, the dimer cluster model), two chains each plus one grown from a zero cutoff."""
    c = CASES[case]
    flat = S.flatten_model(c["model"](S))
    mid = eng.register_model(flat)
    streams = list(c["streams"]) + [99]
    params = [dict(T=c["T"], seed=c["seed"], stream=s, thermalization=c["therm"],
                   init_opstring_cutoff=0 if s == 99 else -1) for s in streams]
    ids = eng.create_walkers(mid, params)
    eng.init(ids)
    eng.sweep(ids, c["therm"] + 6, measure=True)
    om = O.OracleModel(flat)
    for p, wid in zip(params, ids.tolist()):
        w = O.OracleWalker(om, T=p["T"], seed=p["seed"], stream=p["stream"], thermalization=p["thermalization"])
        w.init(init_cutoff=p["init_opstring_cutoff"])
        w.run(c["therm"] + 6, measure=True)
        compare(eng, flat, wid, w)


def square(S, side):
    return S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (side, side)},
                                          "J": 1.0, "measure": ["magnetization", "staggered_magnetization"]}))


def oracle_after(O, flat, p, sweeps, init_cutoff=-1):
    w = O.OracleWalker(O.OracleModel(flat), T=p["T"], seed=p["seed"], stream=p["stream"],
                       thermalization=p.get("thermalization", 0))
    w.init(init_cutoff=init_cutoff)
    w.run(sweeps, measure=True)
    return w


@pytest.mark.parametrize("stage", [0, 4096, 192 * 1024])
def test_emulated_launch_paths_match_oracle(S, O, eng, stage):
    """Batched, one-launch-per-walker (plain) and cost-balanced (sse_sweep_each) launches, with the
    worm update's records in global memory or staged in shared memory: the same chains."""
    flat = square(S, 6)
    mid = eng.register_model(flat)
    params = [dict(T=0.25, seed=31, stream=k, thermalization=4) for k in range(3)]
    ids = eng.create_walkers(mid, params)
    eng.init(ids)
    eng.set_staging(stage)
    try:
        eng.sweep(ids, 5, measure=True)
        eng.sweep(ids[:2], 2, measure=True, plain=True)
        eng.sweep_each(ids, [1, 3, 2], measure=True)
    finally:
        eng.set_staging(0)
    for p, wid, n in zip(params, ids.tolist(), (8, 10, 7)):
        compare(eng, flat, wid, oracle_after(O, flat, p, n))


def test_emulated_export_import_continues_the_chain(S, O, eng):
    """A walker exported mid-chain and imported into a fresh walker sweeps on exactly like the oracle."""
    flat = square(S, 4)
    mid = eng.register_model(flat)
    p = dict(T=0.5, seed=41, stream=3, thermalization=2)
    (a,) = eng.create_walkers(mid, [p]).tolist()
    eng.init([a])
    eng.sweep([a], 6, measure=True)
    ops, st, inf = eng.export(a)
    (b,) = eng.create_walkers(mid, [p]).tolist()
    eng.import_(b, ops, st, inf)
    eng.sweep([b], 5, measure=False)
    w = oracle_after(O, flat, p, 6)
    w.run(5, measure=False)
    compare(eng, flat, b, w, measured=False, counters=False)


def test_emulated_sweep_tempering_matches_oracle(S, O, eng):
    """Blocks of Carlo steps with device exchange steps between them (k_tempering): accept counts,
    temperatures and the accumulators that move with them, as the oracle's exchange gives them."""
    flat = square(S, 4)
    mid = eng.register_model(flat)
    temps, nl, seed = [0.3, 0.45, 0.7, 1.1, 1.7], 3, 41
    nr = len(temps)
    params = [dict(T=temps[k], seed=seed, stream=l * nr + k, thermalization=3) for l in range(nl) for k in range(nr)]
    ids = eng.create_walkers(mid, params).reshape(nl, nr)
    eng.init(ids.ravel())
    om = O.OracleModel(flat)
    ws = []
    for p in params:
        w = O.OracleWalker(om, T=p["T"], seed=seed, stream=p["stream"], thermalization=3)
        w.init()
        ws.append(w)
    nblocks, interval = 10, 3
    acc, prop = eng.sweep_tempering(ids, nblocks, interval, seed=77, first_step=5, measure=True)
    acc_o, prop_o = np.zeros_like(acc), np.zeros_like(prop)
    for b in range(nblocks):
        for w in ws:
            w.run(interval, measure=True)
        a, rc = O.tempering_exchange(ws, nl, nr, seed=77, step=5 + b)
        assert rc == 0
        acc_o += a == 1
        prop_o += a >= 0
    assert np.array_equal(acc, acc_o) and np.array_equal(prop, prop_o) and acc.sum() > 0
    for wid, w in zip(ids.ravel().tolist(), ws):
        assert eng.info(wid)["T"] == w.w.T
        compare(eng, flat, wid, w)


def test_emulated_invariant_check_finds_planted_inconsistency(S, O, eng):
    """k_check passes consistent walkers and reports a spin flipped against the opstring."""
    import sse_gb300.util as U

    flat = square(S, 4)
    mid = eng.register_model(flat)
    a, b = eng.create_walkers(mid, [dict(T=0.5, seed=2, stream=k) for k in range(2)]).tolist()
    eng.init([a, b])
    eng.sweep([a, b], 4)
    assert eng.check([a, b]).tolist() == [0, 0]
    ops, st, inf = eng.export(b)
    site = int(flat.arrays["bond_sites"][2 * U.dev_get_bond(int(ops[np.flatnonzero(ops)[0]]))])
    st = st.copy()
    st[site] ^= 1
    eng.import_(b, ops, st, inf)
    res = eng.check([a, b]).tolist()
    assert res[0] == 0 and res[1] in (4, 5)


def test_emulated_worm_cap_stop_matches_oracle(S, O, eng):
    """The long worm of the S=1 bilayer pinned in test_worm_cap.py, in a measured sweep under the
    lowered cap of that file: the engine's kernels stop the walker where the oracle does, with the same opstring and replay
    counter, while the other walker of the launch completes its sweeps."""
    from sse_gb300.engine import SSEError
    from test_worm_cap import FACTOR, LONG_WORM, MEASURED, long_worm_model

    flat = long_worm_model(S)
    mid = eng.register_model(flat)
    params = [dict(T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=s, thermalization=MEASURED)
              for s in (LONG_WORM["stream"], 0)]
    ids = eng.create_walkers(mid, params)
    eng.set_worm_cap(ids, FACTOR)
    eng.init(ids)
    with pytest.raises(SSEError) as err:
        eng.sweep(ids, 3, measure=False)
    assert err.value.code == 8
    w = O.OracleWalker(O.OracleModel(flat), T=params[0]["T"], seed=params[0]["seed"], stream=params[0]["stream"],
                       thermalization=MEASURED)
    w.w.worm_cap_factor = FACTOR
    w.init()
    with pytest.raises(RuntimeError):
        w.run(3, measure=False)
    compare(eng, flat, int(ids[0]), w, measured=False)
    assert eng.info(int(ids[0]))["worm_undos"] == 0
    assert eng.info(int(ids[1]))["sweeps"] == 3 and eng.info(int(ids[1]))["status"] == 0


@pytest.mark.parametrize("stage,therm", [(0, None), (192 * 1024, None), (0, 1)])
def test_emulated_worm_cap_undo_matches_oracle(S, O, eng, stage, therm):
    """The same worm in a thermalisation sweep: the kernels undo the sweep's worm phase exactly as
    the oracle does (records in global memory, and staged in shared memory), and the walker sweeps
    on bit for bit.  With thermalization = 1 the long worm falls in the last thermalisation sweep
    (sweeps == thermalization): its worm phase is undone with the controller still active, and that
    sweep is nevertheless measured, on the opstring the diagonal update left."""
    from test_worm_cap import FACTOR, LONG_WORM, THERMALISING, long_worm_model

    therm = THERMALISING if therm is None else therm
    measured = therm < THERMALISING
    flat = long_worm_model(S)
    mid = eng.register_model(flat)
    params = [dict(T=1 / LONG_WORM["beta"], seed=LONG_WORM["seed"], stream=s, thermalization=therm)
              for s in (LONG_WORM["stream"], 0)]
    ids = eng.create_walkers(mid, params)
    eng.set_worm_cap(ids, FACTOR)
    eng.init(ids)
    eng.set_staging(stage)
    try:
        eng.sweep(ids, 5, measure=measured)
    finally:
        eng.set_staging(0)
    om = O.OracleModel(flat)
    for p, wid in zip(params, ids.tolist()):
        w = O.OracleWalker(om, T=p["T"], seed=p["seed"], stream=p["stream"], thermalization=therm)
        w.w.worm_cap_factor = FACTOR
        w.init()
        w.run(5, measure=measured)
        compare(eng, flat, wid, w, measured=measured)
        assert eng.info(wid)["worm_undos"] == w.w.worm_undos
    assert eng.info(int(ids[0]))["worm_undos"] == 1
    assert eng.check(ids).tolist() == [0, 0]


def test_emulated_noalloc_matches_oracle(S, O, emu):
    """The allocation-free entry point (k_noalloc_prep, k_walk on its static scratch,
    k_noalloc_finish) against the oracle: two calls of 4 Carlo steps each, the first with an opstring
    buffer too small for the cutoff growth, which returns SSE_ERR_CAPACITY with the size needed and
    resumes when called again with a larger buffer.  On the emulated runtime device addresses are
    host addresses, so numpy buffers are the caller's device memory."""
    import ctypes as C

    from sse_gb300.engine import SSE_SWEEP_MEASURE, NoAllocWalker, device_model_desc

    flat = S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (8, 8)},
                                          "J": 1.0, "measure": ["magnetization", "staggered_magnetization"]}))
    params = dict(T=0.5, seed=4242, stream=17, thermalization=2)
    keep = {}

    def dev(name, arr):
        keep[name] = np.ascontiguousarray(arr).copy()
        return keep[name].ctypes.data

    desc = device_model_desc(flat, dev)
    w = NoAllocWalker(T=params["T"], seed=params["seed"], stream=params["stream"], init_opstring_cutoff=-1,
                      diagonal_warmup_sweeps=5, phase=0, init_num_worms=5.0, num_worms_attenuation_factor=0.01,
                      target_worm_length_fraction=2.0, thermalization=params["thermalization"])
    nobs = 6 + 5 * flat.nest
    state = np.zeros(flat.nsites, dtype=np.uint8)
    osum, ocnt, olast = np.zeros(nobs), np.zeros(nobs, dtype=np.int64), np.zeros(nobs)

    def call(ops, nsweeps):
        return emu.sse_sweep_noalloc(C.byref(desc), C.c_void_p(C.addressof(w)), C.c_void_p(ops.ctypes.data),
                                     len(ops), C.c_void_p(state.ctypes.data), C.c_void_p(osum.ctypes.data),
                                     C.c_void_p(ocnt.ctypes.data), C.c_void_p(olast.ctypes.data), nsweeps,
                                     SSE_SWEEP_MEASURE)

    ops = np.zeros(64, dtype=np.uint32)
    rc = call(ops, 4)
    grown = 0
    while rc == 3:  # SSE_ERR_CAPACITY: the caller grows the opstring, keeping its prefix
        assert w.need_capacity > len(ops)
        bigger = np.zeros(w.need_capacity + 64, dtype=np.uint32)
        bigger[: w.L] = ops[: w.L]
        ops = bigger
        grown += 1
        rc = call(ops, 4 - (w.sweeps if w.phase == 2 else 0))
    assert rc == 0 and grown > 0 and w.sweeps == 4
    assert call(ops, 4) == 0
    o = O.OracleWalker(O.OracleModel(flat), T=params["T"], seed=params["seed"], stream=params["stream"],
                       thermalization=params["thermalization"])
    o.init()
    o.run(8, measure=True)
    assert w.status == 0 and w.L == o.w.L and w.num_operators == o.w.num_operators and w.sweeps == 8
    assert w.rng_counter == o.w.ctr and w.num_worms == o.w.num_worms and w.avg_worm_length == o.w.avg_worm_length
    assert np.array_equal(ops[: w.L], o.ops) and np.array_equal(state, o.state)
    so, co, _ = o.obs()
    assert np.array_equal(ocnt, co)
    np.testing.assert_array_equal(osum, so)


def test_emulated_headline_size_walker_matches_oracle(S, O, eng):
    """One walker of the benchmark workload at full size (32x32 S=1/2 Heisenberg, beta = 16,
    L = 51,154 slots): 12 Carlo steps on emulated warps equal the oracle bit for bit."""
    c = CASES["square32_beta16"]
    flat = S.flatten_model(c["model"](S))
    mid = eng.register_model(flat)
    p = dict(T=c["T"], seed=c["seed"], stream=c["streams"][0], thermalization=c["therm"])
    ids = eng.create_walkers(mid, [p])
    eng.init(ids)
    eng.sweep(ids, c["therm"] + c["sweeps"], measure=True)
    w = O.OracleWalker(O.OracleModel(flat), T=p["T"], seed=p["seed"], stream=p["stream"],
                       thermalization=p["thermalization"])
    w.init()
    w.run(c["therm"] + c["sweeps"], measure=True)
    compare(eng, flat, int(ids[0]), w)
    assert w.w.L > 50_000


def test_emulated_graph_replay_matches_oracle(S, O, eng):
    """Sweep blocks captured once as a CUDA graph (flag and queue resets plus the persistent launch)
    and replayed: the same chains as the oracle, block after block."""
    flat = square(S, 6)
    mid = eng.register_model(flat)
    params = [dict(T=0.3, seed=51, stream=k, thermalization=3) for k in range(3)]
    ids = eng.create_walkers(mid, params)
    eng.init(ids)
    for _ in range(3):  # the first call captures, the others replay the captured graph
        eng.sweep(ids, 2, measure=True, graph=True)
    for p, wid in zip(params, ids.tolist()):
        compare(eng, flat, wid, oracle_after(O, flat, p, 6))


@pytest.mark.parametrize("spin,size", [(1.5, (2, 3)), (2.0, (2, 2))])
def test_emulated_higher_spin_matches_oracle(S, O, eng, spin, size):
    """Site dimensions 4 and 5 (S = 3/2 and 2, with a field; up to 57 vertices and 4 worm types
    per bond type): the kernels' chains equal the oracle's."""
    flat = S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": size}, "S": spin,
                                          "J": 1.0, "hz": 0.1, "measure": S.all_magnetization_estimators(2)}))
    mid = eng.register_model(flat)
    params = [dict(T=0.5, seed=61, stream=k, thermalization=5) for k in range(3)]
    ids = eng.create_walkers(mid, params)
    eng.init(ids)
    eng.sweep(ids, 30, measure=True)
    for p, wid in zip(params, ids.tolist()):
        compare(eng, flat, wid, oracle_after(O, flat, p, 30))


@pytest.mark.parametrize("family", ["square_s1_field", "triangle_xxz"])
def test_emulated_other_families_match_oracle(S, O, eng, family):
    """The S=1 square lattice with a field and single-ion anisotropy, and the frustrated triangular
    XXZ magnet (negative vertex weights, so signed measurements): the kernels' chains equal the
    oracle's."""
    from test_tables import families

    flat = S.flatten_model(families(S)[family](S))
    mid = eng.register_model(flat)
    params = [dict(T=0.5, seed=71, stream=k, thermalization=4) for k in range(3)]
    ids = eng.create_walkers(mid, params)
    eng.init(ids)
    eng.sweep(ids, 20, measure=True)
    for p, wid in zip(params, ids.tolist()):
        compare(eng, flat, wid, oracle_after(O, flat, p, 20))
