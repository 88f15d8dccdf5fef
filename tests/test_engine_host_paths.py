"""The C ABI's host paths without a GPU: the engine library built against a fake CUDA runtime
(tests/fake_cuda), whose device memory is host memory and whose kernel launches do nothing.

What is checked is resource handling on failure.  At every allocation of a registration, a walker
creation, a regrowth and a launch's work buffers, an out-of-memory error is injected.  The call
must then return its error and leave the engine as it was: no allocation leaked, no id handed out,
nothing freed twice, and the next call working.  Validation errors must likewise free what was
already uploaded.  The device code itself is checked on a GPU against the oracle; here it never
runs.
"""

import numpy as np
import pytest

NOMEM, ARG = 6, 1


@pytest.fixture
def eng(fake):
    from sse_gb300.engine import Engine

    fake.fake_cuda_fail_alloc_in(-1)
    e = Engine(0, library=fake)
    yield e
    fake.fake_cuda_fail_alloc_in(-1)
    e.close()


def square(S, side=4):
    return S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (side, side)},
                                          "J": 1.0, "measure": ["magnetization"]}))


def walker_params(n, T=0.5):
    return [dict(T=T, seed=3, stream=k) for k in range(n)]


def allocations_of(fake, call):
    """How many device allocations `call` makes when nothing fails."""
    a0 = fake.fake_cuda_allocs()
    call()
    return fake.fake_cuda_allocs() - a0


def test_lifecycle_frees_every_allocation(S, fake):
    from sse_gb300.engine import Engine

    live0, bad0 = fake.fake_cuda_live_allocs(), fake.fake_cuda_bad_frees()
    e = Engine(0, library=fake)
    mid = e.register_model(square(S))
    ids = e.create_walkers(mid, walker_params(3))
    e.init(ids)
    e.sweep(ids, 2)
    e.reserve(ids[:1], 5000)
    e.destroy_walkers(ids[1:])
    e.close()
    assert fake.fake_cuda_live_allocs() == live0 and fake.fake_cuda_bad_frees() == bad0
    assert fake.fake_cuda_launches() > 0


def test_register_out_of_memory_at_every_allocation(S, fake):
    """Including the engine's first model array: a failed registration leaves no model behind, so
    the next one gets id 0."""
    from sse_gb300.engine import Engine, SSEError

    flat = square(S)
    probe = Engine(0, library=fake)
    n = allocations_of(fake, lambda: probe.register_model(flat))
    probe.close()
    assert n > 10
    for k in range(n):
        e = Engine(0, library=fake)
        live0, bad0 = fake.fake_cuda_live_allocs(), fake.fake_cuda_bad_frees()
        fake.fake_cuda_fail_alloc_in(k)
        with pytest.raises(SSEError) as err:
            e.register_model(flat)
        assert err.value.code == NOMEM, k
        assert fake.fake_cuda_live_allocs() == live0 and fake.fake_cuda_bad_frees() == bad0, k
        assert e.register_model(flat) == 0, k
        e.close()


def test_model_array_growth_out_of_memory_keeps_registered_models(S, fake):
    """The ninth model outgrows the engine's model array.  Whichever allocation of that registration
    fails, the eight models stay registered and usable and the ninth gets id 8 afterwards."""
    from sse_gb300.engine import Engine, SSEError

    flat = square(S)

    def with_eight():
        e = Engine(0, library=fake)
        assert [e.register_model(flat) for _ in range(8)] == list(range(8))
        return e

    probe = with_eight()
    n = allocations_of(fake, lambda: probe.register_model(flat))
    probe.close()
    for k in range(n):
        e = with_eight()
        live0, bad0 = fake.fake_cuda_live_allocs(), fake.fake_cuda_bad_frees()
        fake.fake_cuda_fail_alloc_in(k)
        with pytest.raises(SSEError) as err:
            e.register_model(flat)
        assert err.value.code == NOMEM, k
        assert fake.fake_cuda_live_allocs() == live0 and fake.fake_cuda_bad_frees() == bad0, k
        ids = e.create_walkers(0, walker_params(2))
        e.init(ids)
        e.sweep(ids, 1)
        assert e.register_model(flat) == 8, k
        e.close()


def test_invalid_model_frees_what_was_uploaded(S, eng, fake):
    from sse_gb300.engine import SSEError

    flat = square(S)
    for field, value in (("out_worm", 5), ("out_target", 2 * 60), ("leg_state", 7)):
        bad = square(S)
        bad.arrays = {k: v.copy() for k, v in flat.arrays.items()}
        bad.arrays[field][0] = value
        live0 = fake.fake_cuda_live_allocs()
        with pytest.raises(SSEError) as err:
            eng.register_model(bad)
        assert err.value.code == ARG
        assert fake.fake_cuda_live_allocs() == live0, field
    assert eng.register_model(flat) == 0


def test_walker_creation_out_of_memory_at_every_allocation(S, eng, fake):
    """A failed creation hands out no ids and keeps nothing; the next creation starts at the same id."""
    from sse_gb300.engine import SSEError

    mid = eng.register_model(square(S))
    first = eng.create_walkers(mid, walker_params(1))
    n = allocations_of(fake, lambda: eng.destroy_walkers(eng.create_walkers(mid, walker_params(3))))
    assert n >= 3 * 8
    for k in range(n):
        live0, bad0 = fake.fake_cuda_live_allocs(), fake.fake_cuda_bad_frees()
        fake.fake_cuda_fail_alloc_in(k)
        with pytest.raises(SSEError) as err:
            eng.create_walkers(mid, walker_params(3))
        assert err.value.code == NOMEM, k
        assert fake.fake_cuda_live_allocs() == live0 and fake.fake_cuda_bad_frees() == bad0, k
    fake.fake_cuda_fail_alloc_in(-1)
    ids = eng.create_walkers(mid, walker_params(3))
    assert ids.tolist() == [int(first[0]) + 4, int(first[0]) + 5, int(first[0]) + 6]
    eng.init(np.concatenate([first, ids]))
    assert [eng.info(int(i))["status"] for i in ids] == [0, 0, 0]


def test_walker_creation_with_bad_parameters_allocates_nothing(S, eng, fake):
    from sse_gb300.engine import SSEError

    mid = eng.register_model(square(S))
    a = eng.create_walkers(mid, walker_params(1))
    a0 = fake.fake_cuda_allocs()
    params = walker_params(3)
    params[2]["T"] = 0.0
    with pytest.raises(SSEError) as err:
        eng.create_walkers(mid, params)
    assert err.value.code == ARG and fake.fake_cuda_allocs() == a0
    assert eng.create_walkers(mid, walker_params(1)).tolist() == [int(a[0]) + 1]


def test_destroy_checks_every_id_before_freeing(S, eng, fake):
    from sse_gb300.engine import SSEError

    mid = eng.register_model(square(S))
    a, b = eng.create_walkers(mid, walker_params(2)).tolist()
    live0 = fake.fake_cuda_live_allocs()
    for bad in ([a, 999], [a, b, a], [-1]):
        with pytest.raises(SSEError) as err:
            eng.destroy_walkers(np.array(bad, dtype=np.int32))
        assert err.value.code == ARG
        assert fake.fake_cuda_live_allocs() == live0, bad
        assert eng.info(a)["status"] == 0 and eng.info(b)["status"] == 0
    eng.destroy_walkers(np.array([a], dtype=np.int32))
    with pytest.raises(SSEError):
        eng.info(a)
    eng.info(b)


def test_regrowth_out_of_memory_keeps_the_walker(S, eng, fake):
    from sse_gb300.engine import SSEError

    mid = eng.register_model(square(S))
    (w,) = eng.create_walkers(mid, walker_params(1)).tolist()
    cap0 = eng.info(w)["capacity"]
    for k in range(3):  # the opstring, record and slot-index arrays
        live0 = fake.fake_cuda_live_allocs()
        fake.fake_cuda_fail_alloc_in(k)
        with pytest.raises(SSEError) as err:
            eng.reserve([w], 100_000)
        assert err.value.code == NOMEM
        assert fake.fake_cuda_live_allocs() == live0 and eng.info(w)["capacity"] == cap0, k
    eng.reserve([w], 100_000)
    assert eng.info(w)["capacity"] >= 100_000


def test_work_buffer_growth_out_of_memory_keeps_the_old_buffers(S, eng, fake):
    """A launch over more walkers than ever before grows the work buffers; when that fails, the
    buffers of the earlier, smaller launches are still there for the next one."""
    from sse_gb300.engine import SSEError

    mid = eng.register_model(square(S))
    few = eng.create_walkers(mid, walker_params(4))
    eng.init(few)
    eng.sweep(few, 1)
    many = np.concatenate([few, eng.create_walkers(mid, walker_params(300))])
    for k in range(3):  # the three work buffers
        fake.fake_cuda_fail_alloc_in(k)
        with pytest.raises(SSEError) as err:
            eng.init(many)
        assert err.value.code == NOMEM
        eng.sweep(few, 1)  # right after the failure: the small launch still has its buffers
    eng.init(many)
    eng.sweep(many, 1)
