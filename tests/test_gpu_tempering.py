"""Parallel tempering on the GPU engine against the CPU oracle, through the C ABI
(sse_walker_set_T, sse_tempering_exchange, sse_sweep_tempering; src/sse.jl:390-405)."""

import numpy as np
import pytest

from ed import ed_observables

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module")
def eng():
    from sse_gb300.engine import Engine

    e = Engine(0)
    yield e
    e.close()


def sq4(S):
    return S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (4, 4)}, "J": 1.0,
                          "measure": ["magnetization", "staggered_magnetization"]})


def same_walker(eng, wid, w):
    ops, st, inf = eng.export(wid)
    assert inf["T"] == w.w.T
    assert inf["num_operators"] == w.w.num_operators and inf["L"] == w.w.L
    assert inf["rng_counter"] == w.w.ctr
    assert np.array_equal(ops, w.ops) and np.array_equal(st, w.state)
    s, c, last = eng.observables([wid])[0]
    so, co, lo = w.obs()
    assert np.array_equal(c, co)
    np.testing.assert_allclose(s, so, rtol=RTOL, atol=0)
    np.testing.assert_allclose(last, lo, rtol=RTOL, atol=0)


def make(eng, O, flat, temps, nl, seed, therm=4):
    mid = eng.register_model(flat)
    nr = len(temps)
    params = [dict(T=temps[k], seed=seed, stream=l * nr + k, thermalization=therm) for l in range(nl) for k in range(nr)]
    ids = eng.create_walkers(mid, params).reshape(nl, nr)
    eng.init(ids.ravel())
    om = O.OracleModel(flat)
    ws = []
    for p in params:
        w = O.OracleWalker(om, T=p["T"], seed=seed, stream=p["stream"], thermalization=therm)
        w.init()
        ws.append(w)
    return ids, om, ws


def test_gpu_sweep_tempering_matches_oracle(S, O, eng):
    flat = S.flatten_model(sq4(S))
    temps = [0.3, 0.45, 0.7, 1.1, 1.7]
    ids, om, ws = make(eng, O, flat, temps, nl=3, seed=41)
    nblocks, interval = 10, 3
    acc, prop = eng.sweep_tempering(ids, nblocks, interval, seed=77, first_step=5, measure=True)
    acc_o = np.zeros_like(acc)
    prop_o = np.zeros_like(prop)
    for b in range(nblocks):
        for w in ws:
            w.run(interval, measure=True)
        a, rc = O.tempering_exchange(ws, 3, 5, seed=77, step=5 + b)
        assert rc == 0
        acc_o += a == 1
        prop_o += a >= 0
    assert np.array_equal(acc, acc_o) and np.array_equal(prop, prop_o)
    assert acc.sum() > 0  # some swaps happened
    for wid, w in zip(ids.ravel().tolist(), ws):
        same_walker(eng, wid, w)


def test_gpu_single_exchange_flags_match_oracle(S, O, eng):
    flat = S.flatten_model(sq4(S))
    temps = [0.25, 0.3, 0.36, 0.43]
    ids, om, ws = make(eng, O, flat, temps, nl=4, seed=8)
    eng.sweep(ids.ravel(), 6)
    for w in ws:
        w.run(6)
    # list each ladder's walkers in a shuffled order: ranking is by T
    rng = np.random.default_rng(0)
    perm = np.array([rng.permutation(4) for _ in range(4)])
    shuffled = np.take_along_axis(ids, perm, axis=1)
    ws_sh = [ws[l * 4 + k] for l in range(4) for k in perm[l]]
    for step in range(4):
        a = eng.tempering_exchange(shuffled, seed=123, step=step)
        ao, rc = O.tempering_exchange(ws_sh, 4, 4, seed=123, step=step)
        assert rc == 0 and np.array_equal(a, ao)
    for wid, w in zip(ids.ravel().tolist(), ws):
        assert eng.info(wid)["T"] == w.w.T


def test_gpu_set_T_then_sweep_matches_oracle(S, O, eng):
    flat = S.flatten_model(sq4(S))
    mid = eng.register_model(flat)
    (wid,) = eng.create_walkers(mid, [dict(T=0.5, seed=19, stream=0, thermalization=2)])
    eng.init([wid])
    w = O.OracleWalker(O.OracleModel(flat), T=0.5, seed=19, stream=0, thermalization=2)
    w.init()
    eng.sweep([wid], 5)
    w.run(5)
    eng.set_T(int(wid), 0.8)
    w.w.T = 0.8
    eng.sweep([wid], 7)
    w.run(7)
    same_walker(eng, int(wid), w)


def test_gpu_tempering_argument_errors(S, O, eng):
    from sse_gb300.engine import SSEError

    flat = S.flatten_model(sq4(S))
    mid = eng.register_model(flat)
    ids = eng.create_walkers(mid, [dict(T=t, seed=1, stream=k) for k, t in enumerate([0.5, 0.5, 0.7, 0.9])])
    eng.init(ids)
    with pytest.raises(SSEError):  # equal temperatures in a ladder
        eng.tempering_exchange(ids[:3].reshape(1, 3), seed=0, step=0)
    with pytest.raises(SSEError):  # a walker in two ladders
        eng.tempering_exchange(np.array([[ids[2], ids[3]], [ids[3], ids[2]]]), seed=0, step=0)
    other = eng.register_model(S.flatten_model(S.MagnetModel(
        {"lattice": {"unitcell": S.UnitCells.square, "size": (2, 2)}, "J": 1.0})))
    (x,) = eng.create_walkers(other, [dict(T=0.6, seed=1, stream=9)])
    with pytest.raises(SSEError):  # mixed models
        eng.tempering_exchange(np.array([[ids[2], x]]), seed=0, step=0)
    with pytest.raises(SSEError):
        eng.set_T(int(ids[0]), -1.0)
    # nothing changed
    assert [eng.info(int(i))["T"] for i in ids] == [0.5, 0.5, 0.7, 0.9]


def test_gpu_tempering_mc_matches_ed(S, eng):
    """TemperingMC on the 2x4 square job of the reference's ED tests: every temperature of the ladder
    within |z| <= 4 of exact diagonalisation."""
    from sse_gb300.mc import TemperingMC

    params = {"model": S.MagnetModel, "lattice": {"unitcell": S.UnitCells.square, "size": (2, 4)}, "J": 1.23,
              "hz": -0.2, "measure": S.all_magnetization_estimators(2), "T": 1.0, "seed": 5, "thermalization": 500}
    temps = [0.4, 0.6, 0.9, 1.35]
    pt = TemperingMC(params, temps, nladders=16, interval=5, engine=eng)
    pt.run(sweeps=4000, binsize=250)
    ed = ed_observables(S, pt.model, temps)
    res = pt.results()
    bad = []
    for t, T in enumerate(temps):
        for name in ("Energy", "SpecificHeat", "Mag2", "MagChi"):
            mc, err = res[t][name]
            ref = float(ed[name][t])
            z = abs(mc - ref) / (err if err else 1e-8)
            if z > 4:
                bad.append((T, name, mc, err, ref, z))
    assert not bad, bad
    acc = pt.acceptance()
    assert np.all(acc > 0.0) and np.all(acc < 1.0)
