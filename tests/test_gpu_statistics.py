"""Statistical acceptance: a GPU batch against independent oracle chains at equal sweep count.

The acceptance criterion for the batched engine is energy per site within 2 sigma of the reference
at equal sweep count.  The reference (Julia) cannot run here; the oracle is its statement-by-
statement restatement and is itself pinned to exact diagonalisation (tests/test_ed_compare.py).
So: GPU walkers on Philox streams 0..B-1 and oracle chains on disjoint streams, all with the same
thermalisation and measurement sweep counts, are two independent samples of one distribution.
Each chain's mean over its measured sweeps is one sample; the standard error of a batch is the
spread of its chain means over the square root of their number.  Energy per site must agree within
2 sigma (the stated criterion); the other observables within 4 sigma.  The streams are fixed, so
the outcome is reproducible.

* 8x8 S=1/2 Heisenberg at beta = 2 (the single-walker configuration): 512 GPU walkers against 64
  oracle chains, 1000 + 4000 sweeps.
* 32x32 S=1/2 Heisenberg at beta = 16 (the batched configuration): 256 GPU walkers against 16
  oracle chains, 300 + 300 sweeps.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# observable index -> name (the first six, then SignMag..SignMagChi per estimator)
NAMES = {1: "OperatorCount", 4: "SignEnergy", 5: "WormLengthFraction", 8: "SignMag2", 13: "SignStagMag2",
         14: "SignStagMag4"}
ENERGY = 4


def square(S, side):
    return S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (side, side)},
                                          "J": 1.0, "measure": ["magnetization", "staggered_magnetization"]}))


def chain_means(sums, counts):
    """Per-chain means over the measured sweeps, shape (chains, observables)."""
    return np.array(sums) / np.maximum(np.array(counts), 1)


def zscores(a, b):
    ma, mb = a.mean(0), b.mean(0)
    se = np.sqrt(a.var(0, ddof=1) / len(a) + b.var(0, ddof=1) / len(b))
    return (ma - mb) / np.where(se > 0, se, np.inf), ma, mb, se


@pytest.mark.parametrize("side,beta,ngpu,norc,therm,meas", [(8, 2.0, 512, 64, 1000, 4000),
                                                            (32, 16.0, 256, 16, 300, 300)])
def test_gpu_batch_agrees_with_independent_oracle_chains(S, O, side, beta, ngpu, norc, therm, meas):
    from sse_gb300.engine import Engine

    flat = square(S, side)
    seed = 31337
    eng = Engine(0)
    try:
        mid = eng.register_model(flat)
        ids = eng.create_walkers(mid, [dict(T=1.0 / beta, seed=seed, stream=k, thermalization=therm)
                                       for k in range(ngpu)])
        eng.init(ids)
        done = 0
        while done < therm + meas:
            blk = min(500, therm + meas - done)
            eng.sweep(ids, blk, measure=True)
            done += blk
        obs = eng.observables(ids)
        gpu = chain_means([o[0] for o in obs], [o[1] for o in obs])
        assert all(int(o[1][0]) == meas for o in obs)
    finally:
        eng.close()
    om = O.OracleModel(flat)
    chains = [O.OracleWalker(om, T=1.0 / beta, seed=seed, stream=100_000 + k, thermalization=therm)
              for k in range(norc)]
    for w in chains:
        w.init()
    O.run_parallel(om, chains, therm + meas, measure=True, nthreads=min(16, norc))
    orc = chain_means([w.obs()[0] for w in chains], [w.obs()[1] for w in chains])
    z, mg, mo, se = zscores(gpu, orc)
    report = {NAMES[i]: (round(float(mg[i]), 6), round(float(mo[i]), 6), round(float(z[i]), 2)) for i in NAMES}
    assert abs(z[ENERGY]) < 2.0, report
    for i in NAMES:
        assert abs(z[i]) < 4.0, (NAMES[i], report)
