"""Port of test/test_util.jl, test/test_worms.jl and test/test_opercode.jl."""

import random

import numpy as np


def test_split_idx_known_values(S):
    # test/test_util.jl:3-4
    assert S.split_idx((5, 2), 2) == (2, 1)
    assert S.split_idx((5, 2), 6) == (1, 2)


def test_split_join_roundtrip(S):
    dims = (6, 3, 1, 5)
    for i in range(1, int(np.prod(dims)) + 1):
        assert S.join_idx(dims, S.split_idx(dims, i)) == i
    rng = random.Random(1)
    for _ in range(10):
        dims = tuple(rng.randint(1, 400) for _ in range(3))
        for _ in range(10):
            i = rng.randint(1, int(np.prod(dims)))
            assert S.join_idx(dims, S.split_idx(dims, i)) == i


def test_worms_bijection(S):
    # test/test_worms.jl:1-24
    for dim in (2, 4, 8):
        for state_in in range(1, dim + 1):
            outs = []
            for worm in range(1, S.worm_count(dim) + 1):
                so = S.worm_action(worm, state_in, dim)
                assert S.worm_action(S.worm_inverse(worm, dim), so, dim) == state_in
                outs.append(so)
            outs.append(state_in)
            assert sorted(outs) == list(range(1, dim + 1))


def test_opercode_roundtrip():
    # test/test_opercode.jl:1-25, for both the reference and the device layout
    import sse_gb300.util as U

    rng = random.Random(7)
    for _ in range(20):
        bond = rng.randint(1, 100 * 100)
        for _ in range(20):
            vidx = rng.randint(1, 77)
            for diagonal in (True, False):
                v = U.ref_vertex_code(diagonal, vidx)
                assert not U.ref_vertex_isinvalid(v)
                assert U.ref_vertex_isdiagonal(v) == diagonal
                assert U.ref_vertex_idx(v) == vidx
                op = U.ref_opercode(bond, v)
                assert U.ref_get_bond(op) == bond
                assert U.ref_get_vertex(op) == v
                assert op != 0
                dev = U.ref_to_dev(np.array([op], dtype=np.uint64))[0]
                assert U.dev_get_bond(int(dev)) == bond - 1
                assert U.dev_isdiagonal(int(dev)) == diagonal
                assert (U.dev_get_vcode(int(dev)) >> 1) == vidx - 1
                assert U.dev_to_ref(np.array([dev], dtype=np.uint32))[0] == op
    assert U.ref_vertex_isinvalid(U.REF_INVALID_VERTEX)
