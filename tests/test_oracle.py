"""The CPU oracle against the reference's golden vectors and invariants.

* vertex list golden vector      -- test/test_vertex_list.jl:1-30
* opstring consistency invariant -- test/test_sse.jl:5-28, 63-94
* replay stream known answers    -- Philox4x32-10 (Random123 KAT vectors)
"""

import numpy as np
import pytest


def dev_op(bond1, diag, vidx1):
    import sse_gb300.util as U

    return U.dev_opercode(bond1 - 1, U.dev_vertex_code(diag, vidx1 - 1))


def golden_model(S):
    sp, sz = S.spin_operators(2)
    H = np.kron(sz, sz) + 0.5 * (np.kron(sp, sp.T) + np.kron(sp.T, sp))
    vd = S.make_vertex_data((2, 2), H, energy_offset_factor=0.0)
    bonds = [S.SSEBond(1, (1, 2)), S.SSEBond(1, (2, 3)), S.SSEBond(1, (1, 3))]
    sd = S.SSEData([vd], [S.SSESite(2)] * 4, bonds, vd.energy_offset * 3)
    return S.flatten_sse_data(sd, norm_site_count=4)


def ref_pair(leg1, p1):
    return 4 * (p1 - 1) + (leg1 - 1)


GOLDEN_OPS = [0, 0, (1,), 0, (1,), (2,), (3,)]
GOLDEN_VERTICES = {
    3: [(3, 7), (3, 6), (1, 5), (2, 5)],
    5: [(3, 3), (4, 3), (1, 7), (1, 6)],
    6: [(4, 5), (4, 7), (2, 3), (2, 7)],
    7: [(3, 5), (4, 6), (1, 3), (2, 6)],
}
GOLDEN_V_LAST = [(3, 7), (3, 6), (4, 7), None]
GOLDEN_V_FIRST = [(1, 3), (2, 3), (2, 6), None]


def golden_ops():
    return np.array([0 if o == 0 else dev_op(o[0], False, 1) for o in GOLDEN_OPS], dtype=np.uint32)


def golden_expected():
    exp = -np.ones(4 * len(GOLDEN_OPS), dtype=np.int32)
    for p, legs in GOLDEN_VERTICES.items():
        for leg, (l1, p1) in enumerate(legs):
            exp[4 * (p - 1) + leg] = ref_pair(l1, p1)
    vl = np.array([-1 if x is None else ref_pair(*x) for x in GOLDEN_V_LAST], dtype=np.int32)
    vf = np.array([-1 if x is None else ref_pair(*x) for x in GOLDEN_V_FIRST], dtype=np.int32)
    return exp, vf, vl


def test_vertex_list_golden(S, O):
    flat = golden_model(S)
    om = O.OracleModel(flat)
    w = O.OracleWalker(om, T=1.0, seed=1, stream=0)
    w.set_opstring(golden_ops())
    w.make_vertex_list()
    exp, vf, vl = golden_expected()
    assert np.array_equal(w.vertices, exp)
    assert np.array_equal(w.v_first, vf)
    assert np.array_equal(w.v_last, vl)


def test_philox_kat(O):
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]
    # draw layout: even index -> words 0,1 ; odd index -> words 2,3 of block index>>1
    x = O.philox([5, 0, 7, 0], [11, 0])
    assert O.draw(11, 7, 10) == x[0] | (x[1] << 32)
    assert O.draw(11, 7, 11) == x[2] | (x[3] << 32)


def test_tanh_accuracy(O):
    import math

    for x in np.concatenate([np.linspace(-25, 25, 2001), np.geomspace(1e-12, 1, 200)]):
        t = O.tanh(float(x))
        assert abs(t - math.tanh(x)) <= 4e-16 * max(1.0, abs(math.tanh(x)))


def isconsistent(flat, ops, state0):
    """test/test_sse.jl:5-28 on device opcodes."""
    import sse_gb300.util as U

    a = flat.arrays
    state = np.array(state0, dtype=np.int64)
    for op in ops.tolist():
        if op == 0:
            continue
        b = U.dev_get_bond(op)
        t = a["bond_type"][b]
        v = U.dev_get_vcode(op) >> 1
        ls = a["leg_state"][4 * (a["type_vert_off"][t] + v): 4 * (a["type_vert_off"][t] + v) + 4]
        sites = a["bond_sites"][2 * b: 2 * b + 2]
        if not all(state[sites] < a["site_dims"][sites]):
            return False
        if list(state[sites]) != list(ls[:2]):
            return False
        state[sites] = ls[2:]
    return True


def test_sse_mc_consistency_mixed_spins(S, O):
    # test/test_sse.jl:63-94: honeycomb 4x4 with S=1/2 and S=1 sublattices, T=0.1
    params = {"T": 0.1, "measure": [], "parameter_map": {"S": ("S1", "S2")},
              "lattice": {"unitcell": S.UnitCells.honeycomb, "size": (4, 4)}, "J": 1.4, "S1": 0.5, "S2": 1.0}
    m = S.MagnetModel(params)
    flat = S.flatten_model(m)
    om = O.OracleModel(flat)
    w = O.OracleWalker(om, T=0.1, seed=2024, stream=3, thermalization=100)
    w.init()
    for _ in range(1000):
        assert isconsistent(flat, w.ops, w.state)
        w.step(measure=False)
    assert isconsistent(flat, w.ops, w.state)
    assert np.all(w.state < flat.arrays["site_dims"])


def test_worm_traverse_tiny_opstrings(S, O):
    # test/test_sse.jl:30-61: single worms on hand-built opstrings stay consistent
    m = S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (4, 4)}, "J": 1.0})
    flat = S.flatten_model(m)
    om = O.OracleModel(flat)
    dv = flat.arrays["diag_vertex"]
    for seed in range(20):
        for ops in ([dev_op(1, True, (int(dv[2]) >> 1) + 1)], [dev_op(1, True, 1), dev_op(1, True, 1)]):
            w = O.OracleWalker(om, T=0.1, seed=seed, stream=0, init_num_worms=1.0, attenuation=0.0)
            ops = np.array(ops, dtype=np.uint32)
            w.set_opstring(ops)
            import sse_gb300.util as U
            a = flat.arrays
            v = U.dev_get_vcode(int(ops[0])) >> 1
            st = np.zeros(flat.nsites, dtype=np.uint8)
            st[a["bond_sites"][0]] = a["leg_state"][4 * v]
            st[a["bond_sites"][1]] = a["leg_state"][4 * v + 1]
            w.set_state(st)
            w.make_vertex_list()
            w.worm_update(thermalized=True)
            assert isconsistent(flat, w.ops, w.state)


def test_cutoff_growth_rule(S, O):
    # src/sse.jl:138-145: L <- floor(1.5 L + 100) whenever n >= L/2
    m = S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (4, 4)}, "J": 1.0})
    om = O.OracleModel(S.flatten_model(m))
    w = O.OracleWalker(om, T=0.25, seed=9, stream=1)
    w.init(init_cutoff=0, warmup=0)
    assert w.w.L == 0
    w.diagonal_update()
    assert w.w.L == 100
    Ls = [100]
    for _ in range(40):
        n_before, L_before = w.w.num_operators, w.w.L
        w.diagonal_update()
        if n_before >= 0.5 * L_before:
            assert w.w.L == L_before + L_before // 2 + 100
        else:
            assert w.w.L == L_before
        Ls.append(w.w.L)
    assert Ls[-1] > 100
