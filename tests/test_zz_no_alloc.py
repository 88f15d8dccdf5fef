"""The allocation-free entry point, sse_sweep_noalloc, against the engine's own path.

Callers that cannot call cudaMalloc -- code whose device memory belongs to a host
pool (Julia's CUDA.jl, PyTorch's caching allocator) or a latency-critical loop that
cannot take cudaMalloc's implicit synchronisation -- pass every buffer themselves;
the library keeps its scratch in one static device array.  This test allocates the
caller's buffers with PyTorch and checks two consecutive calls (init! + 5 sweeps,
then 5 more sweeps) against sse_walkers_init + sse_sweep on an engine walker with the
same seed: integer state and controller scalars bit for bit, observables to 1e-12.
It lives in its own file, collected last, and needs nothing from the other tests.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def test_noalloc_matches_engine_path(S):
    torch = pytest.importorskip("torch")
    from sse_gb300.engine import (Engine, NoAllocWalker, SSE_SWEEP_MEASURE, device_model_desc, lib,
                                  sweep_noalloc)

    model = S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (8, 8)}, "J": 1.0,
                           "measure": ["magnetization", "staggered_magnetization"]})
    flat = S.flatten_model(model)
    params = dict(T=0.5, seed=4242, stream=17, thermalization=4)

    # reference: the engine's own entry points
    eng = Engine(0)
    mid = eng.register_model(flat)
    (wid,) = eng.create_walkers(mid, [params])
    eng.init([wid])
    eng.sweep([wid], 5, measure=True)
    eng.sweep([wid], 5, measure=True)
    ops_ref, st_ref, inf_ref = eng.export(int(wid))
    obs_ref = eng.observables([int(wid)])[0]

    # caller-owned device buffers
    keep = []

    def dptr(name, arr):
        t = torch.from_numpy(np.ascontiguousarray(arr).copy()).cuda()
        keep.append(t)
        return t.data_ptr()

    desc = device_model_desc(flat, dptr)
    w = NoAllocWalker()
    w.T, w.seed, w.stream, w.init_opstring_cutoff = params["T"], params["seed"], params["stream"], -1
    w.diagonal_warmup_sweeps, w.phase, w.init_num_worms = 5, 0, 5.0
    w.num_worms_attenuation_factor, w.target_worm_length_fraction = 0.01, 2.0
    w.thermalization = params["thermalization"]
    wdev = torch.frombuffer(bytearray(bytes(w)), dtype=torch.uint8).cuda()
    cap = 8192
    ops = torch.zeros(cap, dtype=torch.int32, device="cuda")
    state = torch.zeros(flat.nsites, dtype=torch.uint8, device="cuda")
    nobs = 6 + 5 * flat.nest
    osum = torch.zeros(nobs, dtype=torch.float64, device="cuda")
    ocnt = torch.zeros(nobs, dtype=torch.int64, device="cuda")
    olast = torch.zeros(nobs, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()

    for _ in range(2):
        rc = sweep_noalloc(desc, wdev.data_ptr(), ops.data_ptr(), cap, state.data_ptr(), osum.data_ptr(),
                           ocnt.data_ptr(), olast.data_ptr(), 5, SSE_SWEEP_MEASURE)
        assert rc == 0, rc

    out = NoAllocWalker.from_buffer_copy(bytes(wdev.cpu().numpy()))
    assert out.status == 0
    assert out.L == inf_ref["L"] and out.num_operators == inf_ref["num_operators"]
    assert out.rng_counter == inf_ref["rng_counter"] and out.sweeps == inf_ref["sweeps"]
    assert out.num_worms == inf_ref["num_worms"] and out.avg_worm_length == inf_ref["avg_worm_length"]
    ops_na = ops.cpu().numpy().view(np.uint32)[: out.L]
    assert np.array_equal(ops_na, ops_ref)
    assert np.array_equal(state.cpu().numpy(), st_ref)
    assert np.array_equal(ocnt.cpu().numpy(), obs_ref[1])
    np.testing.assert_allclose(osum.cpu().numpy(), obs_ref[0], rtol=RTOL, atol=0)
    np.testing.assert_allclose(olast.cpu().numpy(), obs_ref[2], rtol=RTOL, atol=0)

    # sizes beyond the static scratch are rejected before any device work
    assert sweep_noalloc(desc, wdev.data_ptr(), ops.data_ptr(), (1 << 18) + 1, state.data_ptr(), osum.data_ptr(),
                         ocnt.data_ptr(), olast.data_ptr(), 1) == 3
    eng.close()
