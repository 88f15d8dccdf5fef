"""Host-side behaviour of the C ABI on the fake CUDA runtime of tests/fake_cuda (no GPU): the
checkpoint round trip through device memory, the checks on imported walker state, and the argument
checks of the tuning, tempering and walker calls.  Kernels do not run here; everything below is
decided on the host before or after a launch."""

import numpy as np
import pytest

ARG = 1
CAPACITY = 3


@pytest.fixture
def eng(fake):
    from sse_gb300.engine import Engine

    fake.fake_cuda_fail_alloc_in(-1)
    e = Engine(0, library=fake)
    yield e
    e.close()


def square(S, side):
    return S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (side, side)},
                                          "J": 1.0, "measure": ["magnetization"]}))


def oracle_chain(O, flat, T, sweeps, stream=0):
    w = O.OracleWalker(O.OracleModel(flat), T=T, seed=21, stream=stream, thermalization=0)
    w.init()
    w.run(sweeps, measure=False)
    return w


def test_checkpoint_round_trip_through_device_memory(S, O, eng):
    """An oracle chain imported into a walker comes back unchanged from export, including an
    opstring longer than the walker's initial capacity (the import grows it)."""
    flat = square(S, 8)
    mid = eng.register_model(flat)
    (wid,) = eng.create_walkers(mid, [dict(T=1 / 16, seed=21, stream=0)]).tolist()
    cap0 = eng.info(wid)["capacity"]
    w = oracle_chain(O, flat, 1 / 16, 30)
    assert w.w.L > cap0
    sc = w.scalars()
    info = dict(num_operators=sc["n"], rng_counter=sc["ctr"], num_worms=sc["num_worms"],
                avg_worm_length=sc["avg_worm_length"], sweeps=sc["sweeps"])
    eng.import_(wid, w.ops, w.state, info)
    ops, st, inf = eng.export(wid)
    assert np.array_equal(ops, w.ops) and np.array_equal(st, w.state)
    assert inf["L"] == sc["L"] and inf["capacity"] >= sc["L"]
    for k, v in info.items():
        assert inf[k] == v, k
    assert inf["status"] == 0


def test_import_rejects_bad_state_and_leaves_the_walker(S, O, eng):
    import sse_gb300.util as U

    flat = square(S, 4)
    mid = eng.register_model(flat)
    (wid,) = eng.create_walkers(mid, [dict(T=0.5, seed=21, stream=0)]).tolist()
    w = oracle_chain(O, flat, 0.5, 10)
    info = dict(num_operators=int(w.w.num_operators), rng_counter=int(w.w.ctr), num_worms=float(w.w.num_worms),
                avg_worm_length=float(w.w.avg_worm_length), sweeps=int(w.w.sweeps))
    eng.import_(wid, w.ops, w.state, info)
    before = eng.export(wid)
    nverts = int(flat.arrays["type_nverts"][0])
    k = int(np.flatnonzero(w.ops)[0])
    bad_vertex = w.ops.copy()
    bad_vertex[k] = U.dev_opercode(U.dev_get_bond(int(w.ops[k])), U.dev_vertex_code(1, nverts))
    bad_bond = w.ops.copy()
    bad_bond[k] = U.dev_opercode(flat.nbonds, U.dev_get_vcode(int(w.ops[k])))
    bad_state = w.state.copy()
    bad_state[0] = 2
    cases = [(bad_vertex, w.state, info), (bad_bond, w.state, info), (w.ops, bad_state, info),
             (w.ops, w.state, dict(info, num_operators=info["num_operators"] + 1))]
    from sse_gb300.engine import SSEError

    for ops, st, inf in cases:
        with pytest.raises(SSEError) as err:
            eng.import_(wid, ops, st, inf)
        assert err.value.code == ARG
        after = eng.export(wid)
        assert np.array_equal(after[0], before[0]) and np.array_equal(after[1], before[1])
        assert after[2]["num_operators"] == before[2]["num_operators"]


def test_walker_call_argument_checks(S, eng):
    from sse_gb300.engine import SSEError

    mid = eng.register_model(square(S, 4))
    a, b = eng.create_walkers(mid, [dict(T=0.5, seed=1, stream=k) for k in range(2)]).tolist()
    eng.init([a, b])
    calls = [
        lambda: eng.sweep([a, b], -1),
        lambda: eng.sweep([a, a], 1),
        lambda: eng.sweep([a, 77], 1),
        lambda: eng.sweep_each([a, b], [1, -1]),
        lambda: eng.set_worm_cap([a], 0),
        lambda: eng.set_T(a, 0.0),
        lambda: eng.set_T(a, -1.0),
        lambda: eng.set_T(77, 0.5),
        lambda: eng.set_staging(-1),
        lambda: eng.set_staging(10**7),
        lambda: eng.info(77),
        lambda: eng.reserve([a], -5),
        lambda: eng.check([a, 77]),
    ]
    for i, call in enumerate(calls):
        with pytest.raises(SSEError) as err:
            call()
        assert err.value.code == ARG, i
    with pytest.raises(ValueError):
        eng.sweep_each([a, b], [1])
    eng.set_staging(1000)
    assert eng.get_staging() == 1024  # rounded up to whole 32-byte records
    eng.set_staging(0)
    eng.set_T(a, 0.25)
    assert eng.info(a)["T"] == 0.25
    # the invariant check only reads walkers, so a walker may be listed twice
    assert eng.check([a, a]).shape == (2,)


def test_destroyed_walkers_are_refused_everywhere(S, O, eng):
    from sse_gb300.engine import SSEError

    flat = square(S, 4)
    mid = eng.register_model(flat)
    a, b = eng.create_walkers(mid, [dict(T=0.5, seed=1, stream=k) for k in range(2)]).tolist()
    eng.init([a, b])
    eng.destroy_walkers([a])
    w = oracle_chain(O, flat, 0.5, 3)
    info = dict(num_operators=int(w.w.num_operators), rng_counter=0, num_worms=5.0, avg_worm_length=1.0, sweeps=0)
    for call in (lambda: eng.info(a), lambda: eng.sweep([a], 1), lambda: eng.init([a]),
                 lambda: eng.observables([a]), lambda: eng.import_(a, w.ops, w.state, info),
                 lambda: eng.destroy_walkers([a]), lambda: eng.set_T(a, 1.0), lambda: eng.check([a])):
        with pytest.raises((SSEError, KeyError)):
            call()
    # ids are never reused
    (c,) = eng.create_walkers(mid, [dict(T=0.5, seed=1, stream=2)]).tolist()
    assert c not in (a, b)
    eng.sweep([b, c], 1)


def test_tempering_ladder_checks(S, eng):
    """A ladder is a (nladders, nrungs >= 2) array of distinct walkers of one model."""
    from sse_gb300.engine import SSEError

    m1 = eng.register_model(square(S, 4))
    m2 = eng.register_model(square(S, 6))
    w1 = eng.create_walkers(m1, [dict(T=0.2 * (k + 1), seed=1, stream=k) for k in range(4)])
    w2 = eng.create_walkers(m2, [dict(T=0.3, seed=1, stream=9)])
    eng.init(np.concatenate([w1, w2]))
    for ladders in ([[w1[0], w1[1]], [w1[1], w1[2]]],  # a walker in two ladders
                    [[w1[0], w2[0]]],                  # two models in one ladder
                    [[w1[0], w1[0]]],                  # a walker twice in one ladder
                    [[w1[0], 99]]):                    # an unknown walker
        with pytest.raises(SSEError) as err:
            eng.tempering_exchange(np.array(ladders, dtype=np.int32), seed=1, step=0)
        assert err.value.code == ARG, ladders
    with pytest.raises(ValueError):
        eng.tempering_exchange(np.array([[w1[0]]], dtype=np.int32), seed=1, step=0)
    acc = eng.tempering_exchange(np.array([[w1[0], w1[1]], [w1[2], w1[3]]], dtype=np.int32), seed=1, step=0)
    assert acc.shape == (2, 1)


def test_noalloc_argument_and_limit_checks(S, fake):
    """sse_sweep_noalloc refuses null buffers and a negative sweep count (SSE_ERR_ARG) and sizes
    beyond its static scratch (SSE_ERR_CAPACITY) before it launches anything.  On the fake runtime
    device addresses are host addresses, so numpy buffers stand in for the caller's device memory."""
    import ctypes as C

    from sse_gb300.engine import SSE_SWEEP_MEASURE, NoAllocWalker, device_model_desc

    CAPACITY = 3
    flat = square(S, 4)
    keep = {}

    def dev(name, arr):
        keep[name] = np.ascontiguousarray(arr)
        return keep[name].ctypes.data

    desc = device_model_desc(flat, dev)
    walker = NoAllocWalker(T=0.5, seed=1, stream=0, init_opstring_cutoff=-1, diagonal_warmup_sweeps=5,
                           init_num_worms=5.0, num_worms_attenuation_factor=0.01, target_worm_length_fraction=2.0)
    ops = np.zeros(256, dtype=np.uint32)
    state = np.zeros(flat.nsites, dtype=np.uint8)
    nobs = 6 + 5 * flat.nest
    obs_sum, obs_last, obs_count = np.zeros(nobs), np.zeros(nobs), np.zeros(nobs, dtype=np.int64)

    def call(d=desc, w=C.addressof(walker), o=ops.ctypes.data, cap=len(ops), s=state.ctypes.data, n=1):
        return fake.sse_sweep_noalloc(C.byref(d), C.c_void_p(w), C.c_void_p(o), cap, C.c_void_p(s),
                                      C.c_void_p(obs_sum.ctypes.data), C.c_void_p(obs_count.ctypes.data),
                                      C.c_void_p(obs_last.ctypes.data), n, SSE_SWEEP_MEASURE)

    launches0 = fake.fake_cuda_launches()
    assert call(w=None) == ARG and call(o=None) == ARG and call(s=None) == ARG and call(n=-1) == ARG
    assert call(cap=0) == CAPACITY and call(cap=(1 << 18) + 1) == CAPACITY
    for field, value, code in (("nsites", (1 << 14) + 1, CAPACITY), ("nbonds", (1 << 16) + 1, CAPACITY),
                               ("ntypes", 65, CAPACITY), ("maxdim", 1, ARG), ("nest", -1, ARG)):
        d = device_model_desc(flat, dev)
        setattr(d, field, value)
        assert call(d=d) == code, field
    assert fake.fake_cuda_launches() == launches0
    assert call() == 0 and fake.fake_cuda_launches() > launches0


def test_walker_creation_refuses_infinite_T_and_oversize_cutoffs(S, eng):
    """Links and slot indices are 32-bit, so opstrings stay below 2^29 slots from creation on; an
    infinite temperature (whose cutoff round(N*T) has no value) is refused like a non-positive one,
    all before anything is allocated."""
    from sse_gb300.engine import SSEError

    mid = eng.register_model(square(S, 4))
    for params, code in [
        (dict(T=float("inf"), seed=1), ARG),
        (dict(T=float("nan"), seed=1), ARG),
        (dict(T=0.5, seed=1, init_opstring_cutoff=1 << 28), CAPACITY),
        (dict(T=2.0 ** 40, seed=1), CAPACITY),  # round(16 T) far above 2^29
    ]:
        with pytest.raises(SSEError) as err:
            eng.create_walkers(mid, [dict(T=0.5, seed=1), params])
        assert err.value.code == code, params
    # a cutoff that fits gets 2 c + 100 slots, rounded up to 64
    (w,) = eng.create_walkers(mid, [dict(T=0.5, seed=1, init_opstring_cutoff=1000)]).tolist()
    assert eng.info(w)["capacity"] >= 2100


def test_worm_counts_out_of_range_are_refused(S, O, eng):
    """A sweep runs ceil(num_worms) worms: an infinite or huge count (created or imported) would keep
    one sweep on the GPU for hours, so both paths refuse it, and import leaves the walker as it was."""
    from sse_gb300.engine import SSEError

    flat = square(S, 4)
    mid = eng.register_model(flat)
    for nw in (float("inf"), float("nan"), -1.0, 2.0 ** 32):
        with pytest.raises(SSEError) as err:
            eng.create_walkers(mid, [dict(T=0.5, seed=1, init_num_worms=nw)])
        assert err.value.code == ARG, nw
    (wid,) = eng.create_walkers(mid, [dict(T=0.5, seed=21, stream=0)]).tolist()
    w = oracle_chain(O, flat, 0.5, 20)
    info = dict(num_operators=int(w.w.num_operators), rng_counter=int(w.w.ctr), num_worms=float(w.w.num_worms),
                avg_worm_length=float(w.w.avg_worm_length), sweeps=int(w.w.sweeps))
    eng.import_(wid, w.ops, w.state, info)
    before = eng.info(wid)
    for key, bad in (("num_worms", float("inf")), ("num_worms", 2.0 ** 40), ("avg_worm_length", float("nan")),
                     ("avg_worm_length", -1.0)):
        with pytest.raises(SSEError) as err:
            eng.import_(wid, w.ops, w.state, dict(info, **{key: bad}))
        assert err.value.code == ARG, (key, bad)
    after = eng.info(wid)
    assert after["num_worms"] == before["num_worms"] and after["avg_worm_length"] == before["avg_worm_length"]
