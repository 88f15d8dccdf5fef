"""The C ABI rejects tables and walker state that would make the sweep kernel index outside its
tables.  Every bad input here is refused on the host with SSE_ERR_ARG before any kernel sees it."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from sse_gb300.engine import Engine

    e = Engine(0)
    yield e
    e.close()


def square(S):
    return S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (4, 4)}, "J": 1.0}))


def copy_flat(flat):
    import copy

    f = copy.copy(flat)
    f.arrays = {k: v.copy() for k, v in flat.arrays.items()}
    return f


def test_register_rejects_leg_state_outside_site(S, eng):
    from sse_gb300.engine import SSEError

    bad = copy_flat(square(S))
    bad.arrays["leg_state"][0] = 7  # spin-1/2 sites have states 0 and 1
    with pytest.raises(SSEError) as err:
        eng.register_model(bad)
    assert err.value.code == 1


def test_register_rejects_outcome_outside_type(S, eng):
    from sse_gb300.engine import SSEError

    bad = copy_flat(square(S))
    bad.arrays["out_worm"][0] = 5  # worm index beyond the type's maxworm
    with pytest.raises(SSEError):
        eng.register_model(bad)
    bad = copy_flat(square(S))
    bad.arrays["out_target"][0] = 2 * 60  # a vertex the type does not have
    with pytest.raises(SSEError):
        eng.register_model(bad)


def test_import_rejects_bad_vertex_and_state(S, eng):
    from sse_gb300.engine import SSEError
    import sse_gb300.util as U

    flat = square(S)
    mid = eng.register_model(flat)
    (wid,) = eng.create_walkers(mid, [dict(T=0.5, seed=1, stream=0)])
    eng.init([wid])
    eng.sweep([wid], 3)
    ops, st, inf = eng.export(int(wid))
    nverts = int(flat.arrays["type_nverts"][0])
    bad_ops = ops.copy()
    k = int(np.flatnonzero(bad_ops)[0])
    bad_ops[k] = U.dev_opercode(U.dev_get_bond(int(bad_ops[k])), U.dev_vertex_code(1, nverts))
    with pytest.raises(SSEError):
        eng.import_(int(wid), bad_ops, st, inf)
    bad_st = st.copy()
    bad_st[0] = 2
    with pytest.raises(SSEError):
        eng.import_(int(wid), ops, bad_st, inf)
    # the walker is untouched and still sweeps
    eng.import_(int(wid), ops, st, inf)
    eng.sweep([wid], 2)
    assert eng.info(int(wid))["status"] == 0


def test_device_check_finds_planted_inconsistency(S, eng):
    """sse_check_walkers reports a spin flipped against the opstring (a valid state value, so
    nothing is indexed out of range); the untouched walker passes."""
    flat = square(S)
    mid = eng.register_model(flat)
    a, b = eng.create_walkers(mid, [dict(T=0.5, seed=2, stream=k) for k in range(2)])
    eng.init([a, b])
    eng.sweep([a, b], 4)
    assert eng.check([a, b]).tolist() == [0, 0]
    ops, st, inf = eng.export(int(b))
    # flip a spin that an operator acts on
    import sse_gb300.util as U

    site = int(flat.arrays["bond_sites"][2 * U.dev_get_bond(int(ops[np.flatnonzero(ops)[0]]))])
    st = st.copy()
    st[site] ^= 1
    eng.import_(int(b), ops, st, inf)
    res = eng.check([a, b]).tolist()
    assert res[0] == 0 and res[1] in (4, 5)


def test_duplicate_walker_ids_rejected(S, eng):
    """Two warps must never run the same chain: a walker listed twice is refused before any launch."""
    from sse_gb300.engine import SSEError

    mid = eng.register_model(square(S))
    a, b = eng.create_walkers(mid, [dict(T=0.5, seed=3, stream=k) for k in range(2)])
    with pytest.raises(SSEError):
        eng.init([a, b, a])
    eng.init([a, b])
    with pytest.raises(SSEError):
        eng.sweep([a, a], 1)
    with pytest.raises(SSEError):
        eng.sweep_each([b, a, b], [1, 1, 1])
    with pytest.raises(SSEError):
        eng.autotune([a, a], nsweeps_probe=1)
    assert [eng.info(int(i))["sweeps"] for i in (a, b)] == [0, 0]
    eng.sweep([a, b], 1)
    assert eng.check([a, b]).tolist() == [0, 0]
