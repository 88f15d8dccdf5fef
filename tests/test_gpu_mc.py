"""The Python mirror of the Carlo interface on the GPU engine: statistics against exact
diagonalisation (check (b)) and the reference checkpoint round trip."""

import numpy as np
import pytest

from ed import ed_observables
from test_ed_compare import JOBS, make_model

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("job", list(JOBS))
@pytest.mark.parametrize("T", [0.04, 0.7, 2.02])
def test_batch_mc_vs_ed(S, job, T):
    p = dict(JOBS[job])
    uc, size = p.pop("lattice")
    p.update(model=S.MagnetModel, T=T, thermalization=1000, seed=124535,
             lattice={"unitcell": getattr(S.UnitCells, uc), "size": size}, measure=S.all_magnetization_estimators(2))
    mc = S.BatchMC(p, nwalkers=64)
    mc.run(sweeps=2000, binsize=500)
    res = mc.results()
    ed = ed_observables(S, make_model(S, JOBS[job]), [T])
    bad = []
    for name, vals in ed.items():
        mean, err = res[name]
        z = abs(mean - vals[0]) / (err if err > 0 else 1e-8)
        if z > 4:
            bad.append((name, mean, err, float(vals[0]), z))
    assert not bad, bad


def test_mc_checkpoint_roundtrip(S):
    params = {"model": S.MagnetModel, "T": 0.3, "thermalization": 5, "seed": 77,
              "lattice": {"unitcell": S.UnitCells.square, "size": (6, 6)}, "J": 1.0, "measure": ["magnetization"]}
    a = S.MC(params, stream=3)
    b = S.MC(params, stream=3)
    ctx_a, ctx_b = S.MCContext(params), S.MCContext(params)
    a.init(ctx_a)
    for _ in range(12):
        a.sweep(ctx_a)
        a.measure(ctx_a)
    ck = a.write_checkpoint()
    assert ck["operators"].dtype == np.uint64 and ck["state"].min() >= 1
    b.read_checkpoint(ck)
    for _ in range(7):
        a.sweep(ctx_a)
        b.sweep(ctx_b)
    ca, cb = a.write_checkpoint(), b.write_checkpoint()
    assert np.array_equal(ca["operators"], cb["operators"]) and np.array_equal(ca["state"], cb["state"])
    assert "SignEnergy" in ctx_a.observables and len(ctx_a.observables["Sign"]) == 12 - 5
