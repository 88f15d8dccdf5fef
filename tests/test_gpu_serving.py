"""The request loop on the GPU: a request's result is the same alone and in a mix."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_request_alone_equals_in_mix(S):
    from sse_gb300.engine import Engine
    from sse_gb300.serving import Request, ServingLoop, draw_requests

    target = Request(999, 0.0, 0.5, "square", 6, 2.0, nwalkers=3, nsweeps=40, seed=31337, thermalization=8)
    e1 = Engine(0)
    alone = ServingLoop(e1, memory_budget=1 << 33, tick_sweeps=7)
    r_alone = [r for r in alone.run([target], realtime=False) if r.rid == 999][0]
    e1.close()

    others = draw_requests(5, 12, rate=1000.0, side=(4, 8), beta=(0.5, 4.0), walkers=(1, 5), sweeps=(10, 60))
    e2 = Engine(0)
    mix = ServingLoop(e2, memory_budget=1 << 33, tick_sweeps=7)
    target_late = Request(999, 0.004, 0.5, "square", 6, 2.0, nwalkers=3, nsweeps=40, seed=31337, thermalization=8)
    res = mix.run(others + [target_late], realtime=False)
    e2.close()
    r_mix = [r for r in res if r.rid == 999][0]
    assert len(res) == 13
    assert np.array_equal(r_alone.counts, r_mix.counts)
    np.testing.assert_allclose(r_alone.sums, r_mix.sums, rtol=0, atol=0)
    assert r_alone.operator_updates == r_mix.operator_updates
