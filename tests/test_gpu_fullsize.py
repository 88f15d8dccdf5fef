"""The benchmark configuration at full size: 4096 walkers of the 32x32 S=1/2 Heisenberg model at
beta = 16 in one batch, checked through properties that do not depend on the batch size:

* sampled walkers equal the oracle bit for bit,
* every sampled opstring is consistent with its spin state and periodic in imaginary time
  (the reference's isconsistent, test/test_sse.jl:5-28), and every walker passes the same check
  on the device,
* every cutoff lies on the reference's growth ladder L <- floor(1.5 L + 100) from round(N T),
* walkers re-run alone end in the same state as in the full batch.
"""

import numpy as np
import pytest

from test_oracle import isconsistent

pytestmark = pytest.mark.gpu

NW, SIDE, BETA, SWEEPS, SEED = 4096, 32, 16.0, 12, 4242


@pytest.fixture(scope="module")
def batch(S):
    from sse_gb300.engine import Engine

    flat = S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (SIDE, SIDE)},
                                          "J": 1.0, "measure": ["magnetization", "staggered_magnetization"]}))
    eng = Engine(0)
    mid = eng.register_model(flat)
    params = [dict(T=1.0 / BETA, seed=SEED, stream=k, thermalization=6) for k in range(NW)]
    ids = eng.create_walkers(mid, params)
    eng.init(ids)
    eng.sweep(ids, SWEEPS, measure=True)
    yield eng, flat, mid, ids
    eng.close()


def growth_ladder(L0, upto):
    out = [L0]
    while out[-1] < upto:
        out.append(out[-1] + out[-1] // 2 + 100)
    return set(out)


def test_fullsize_samples_match_oracle(S, O, batch):
    eng, flat, mid, ids = batch
    om = O.OracleModel(flat)
    rng = np.random.default_rng(1)
    for k in sorted(rng.choice(NW, 3, replace=False).tolist()) + [NW - 1]:
        w = O.OracleWalker(om, T=1.0 / BETA, seed=SEED, stream=k, thermalization=6)
        w.init()
        w.run(SWEEPS, measure=True)
        ops, st, inf = eng.export(int(ids[k]))
        assert inf["status"] == 0 and inf["L"] == w.w.L and inf["rng_counter"] == w.w.ctr
        assert np.array_equal(ops, w.ops) and np.array_equal(st, w.state)
        s, c, _ = eng.observables([int(ids[k])])[0]
        so, co, _ = w.obs()
        assert np.array_equal(c, co)
        np.testing.assert_allclose(s, so, rtol=1e-12, atol=0)


def test_fullsize_opstrings_consistent_and_on_growth_ladder(batch):
    eng, flat, mid, ids = batch
    L0 = int(np.rint(flat.nsites / BETA))
    infos = [eng.info(int(i)) for i in ids]
    Lmax = max(x["L"] for x in infos)
    ladder = growth_ladder(L0, Lmax)
    assert all(x["L"] in ladder and x["status"] == 0 and x["sweeps"] == SWEEPS for x in infos)
    assert all(0 < x["num_operators"] < x["L"] for x in infos)
    rng = np.random.default_rng(2)
    for k in rng.choice(NW, 6, replace=False).tolist():
        ops, st, inf = eng.export(int(ids[k]))
        assert int(np.count_nonzero(ops)) == inf["num_operators"]
        assert isconsistent(flat, ops, st)
        # imaginary-time periodicity: propagating the state through the whole opstring returns it
        import sse_gb300.util as U

        a = flat.arrays
        state = st.astype(np.int64).copy()
        for op in ops[ops != 0].tolist():
            b = U.dev_get_bond(op)
            v = U.dev_get_vcode(op) >> 1
            off = 4 * (a["type_vert_off"][a["bond_type"][b]] + v)
            state[a["bond_sites"][2 * b: 2 * b + 2]] = a["leg_state"][off + 2: off + 4]
        assert np.array_equal(state, st)


def test_fullsize_every_walker_passes_device_invariant_check(batch):
    """isconsistent, periodicity, ranges and operator count for all 4096 walkers (sse_check_walkers)."""
    eng, flat, mid, ids = batch
    res = eng.check(ids)
    assert res.shape == (NW,) and not res.any(), np.bincount(res)


def test_fullsize_walkers_alone_equal_in_batch(batch):
    eng, flat, mid, ids = batch
    rng = np.random.default_rng(3)
    pick = sorted(rng.choice(NW, 5, replace=False).tolist())
    alone = eng.create_walkers(mid, [dict(T=1.0 / BETA, seed=SEED, stream=k, thermalization=6) for k in pick])
    eng.init(alone)
    eng.sweep(alone, SWEEPS, measure=True)
    for k, a in zip(pick, alone.tolist()):
        oa, sa, ia = eng.export(a)
        ob, sb, ib = eng.export(int(ids[k]))
        assert np.array_equal(oa, ob) and np.array_equal(sa, sb) and ia["rng_counter"] == ib["rng_counter"]
        np.testing.assert_array_equal(eng.observables([a])[0][0], eng.observables([int(ids[k])])[0][0])
