"""The allocation-free entry point's input checks, run on emulated warps (tests/warp_emu).

sse_sweep_noalloc takes the model tables and the walker from the caller's device memory, so its
checks run on the device, in k_noalloc_prep, before anything is derived or swept.  Each case below
corrupts one table entry or one walker field that a later kernel would index with, and expects the
call to refuse it (SSE_ERR_ARG, or SSE_ERR_UNSUPPORTED for an over-long transition row) with the
walker's chain -- cutoff, operator count, sweeps, replay counter, opstring -- left as it was.  The
same checks on the engine's host path (sse_model_register) are exercised by the last test.  On the
emulated runtime device addresses are host addresses, so numpy buffers are the caller's memory.
"""

import ctypes as C

import numpy as np
import pytest

ARG, UNSUPPORTED = 1, 9


def square(S, side=4):
    return S.flatten_model(S.MagnetModel({"lattice": {"unitcell": S.UnitCells.square, "size": (side, side)},
                                          "J": 1.0, "measure": ["magnetization"]}))


class Caller:
    """One caller of sse_sweep_noalloc: its model tables (copies that a case may corrupt), walker,
    opstring, spin state and observables, all in 'device' (host) memory."""

    def __init__(self, S, emu, flat, cap=4096):
        from sse_gb300.engine import NoAllocWalker

        self.emu, self.flat = emu, flat
        self.arrays = {k: np.ascontiguousarray(v).copy() for k, v in flat.arrays.items()}
        self.w = NoAllocWalker(T=0.5, seed=7, stream=3, init_opstring_cutoff=-1, diagonal_warmup_sweeps=5, phase=0,
                               init_num_worms=5.0, num_worms_attenuation_factor=0.01,
                               target_worm_length_fraction=2.0, thermalization=1)
        self.ops = np.zeros(cap, dtype=np.uint32)
        self.state = np.zeros(flat.nsites, dtype=np.uint8)
        nobs = 6 + 5 * flat.nest
        self.osum, self.ocnt, self.olast = np.zeros(nobs), np.zeros(nobs, dtype=np.int64), np.zeros(nobs)

    def desc(self):
        from sse_gb300.engine import MODEL_TABLES, device_model_desc

        dt = dict(MODEL_TABLES)
        conv = {k: np.ascontiguousarray(v, dtype=dt[k]) for k, v in self.arrays.items()}
        self._keep = conv

        class F:
            pass

        f = F()
        for k in ("nsites", "nbonds", "ntypes", "maxdim", "nest", "energy_offset", "norm_site_count"):
            setattr(f, k, getattr(self.flat, k))
        f.arrays = conv
        return device_model_desc(f, lambda name, arr: conv[name].ctypes.data)

    def call(self, nsweeps=2):
        from sse_gb300.engine import SSE_SWEEP_MEASURE

        d = self.desc()
        return self.emu.sse_sweep_noalloc(C.byref(d), C.c_void_p(C.addressof(self.w)), C.c_void_p(self.ops.ctypes.data),
                                          len(self.ops), C.c_void_p(self.state.ctypes.data),
                                          C.c_void_p(self.osum.ctypes.data), C.c_void_p(self.ocnt.ctypes.data),
                                          C.c_void_p(self.olast.ctypes.data), nsweeps, SSE_SWEEP_MEASURE)

    def chain(self):
        w = self.w
        return (w.L, w.num_operators, w.sweeps, w.rng_counter, w.phase, self.ops.tobytes(), self.state.tobytes(),
                self.ocnt.tobytes())


def first_offdiagonal_vertex(a):
    ls = a["leg_state"].reshape(-1, 4)
    return int(np.nonzero((ls[:, 0] != ls[:, 2]) | (ls[:, 1] != ls[:, 3]))[0][0])


def first_row_with_outcomes(a):
    return int(np.nonzero(a["trans_start"] >= 0)[0][0])


# table corruptions: (name, function of the arrays, expected status)
TABLE_CASES = [
    ("bond site out of range", lambda a: a["bond_sites"].__setitem__(1, 10**6), ARG),
    ("bond joins a site to itself", lambda a: a["bond_sites"].__setitem__(1, a["bond_sites"][0]), ARG),
    ("bond type out of range", lambda a: a["bond_type"].__setitem__(0, 7), ARG),
    ("leg state outside the site's dimension", lambda a: a["leg_state"].__setitem__(5, 2), ARG),
    ("diagonal vertex code even (an off-diagonal code)", lambda a: a["diag_vertex"].__setitem__(0, 2), ARG),
    ("diagonal vertex index past the type's vertices", lambda a: a["diag_vertex"].__setitem__(0, 2 * 40 + 1), ARG),
    ("diagonal table names an off-diagonal vertex",
     lambda a: a["diag_vertex"].__setitem__(0, 2 * first_offdiagonal_vertex(a) + 1), ARG),
    ("negative vertex offset", lambda a: a["type_vert_off"].__setitem__(1, -6), ARG),
    ("negative diagonal offset", lambda a: a["type_diag_off"].__setitem__(1, -1), ARG),
    ("negative transition offset", lambda a: a["type_trans_off"].__setitem__(1, -24), ARG),
    ("maxworm beyond 8 bits", lambda a: a["type_maxworm"].__setitem__(0, 256), ARG),
    ("two types share transition rows", lambda a: a["type_trans_off"].__setitem__(1, 0), ARG),
    ("outcome target past the type's vertices",
     lambda a: a["out_target"].__setitem__(a["trans_start"][first_row_with_outcomes(a)], 2 * 40), ARG),
    ("outcome worm beyond maxworm",
     lambda a: a["out_worm"].__setitem__(a["trans_start"][first_row_with_outcomes(a)], 2), ARG),
    ("outcome leg out of range",
     lambda a: a["out_leg"].__setitem__(a["trans_start"][first_row_with_outcomes(a)], 4), ARG),
    ("transition row longer than 256 outcomes", lambda a: long_row(a), UNSUPPORTED),
]


def long_row(a):
    """The first row with outcomes gets 300 of them, appended to the outcome tables (so that the
    tables stay as long as the row says)."""
    r = first_row_with_outcomes(a)
    o = a["trans_start"][r]
    a["trans_start"][r], a["trans_count"][r] = len(a["out_cum"]), 300
    for k in ("out_cum", "out_target", "out_leg", "out_worm"):
        a[k] = np.concatenate([a[k], np.repeat(a[k][o:o + 1], 300)])


def extend_tables_with_orphan_row(a):
    """Four rows inserted before the second bond type's rows, the first of them with an outcome: a
    row with outcomes inside the transition table that no bond type's range covers."""
    t1 = int(a["type_trans_off"][1])
    st = a["trans_start"][first_row_with_outcomes(a)]
    a["trans_start"] = np.insert(a["trans_start"], t1, [st, -1, -1, -1]).astype(np.int32)
    a["trans_count"] = np.insert(a["trans_count"], t1, [1, 0, 0, 0]).astype(np.int32)
    a["type_trans_off"][1] = t1 + 4


@pytest.mark.parametrize("name,corrupt,code", TABLE_CASES, ids=[c[0] for c in TABLE_CASES])
def test_noalloc_refuses_bad_tables(S, emu, name, corrupt, code):
    flat = square(S)
    c = Caller(S, emu, flat)
    assert c.call() == 0 and c.w.sweeps == 2  # the intact tables sweep
    before = c.chain()
    corrupt(c.arrays)
    assert c.call() == code, name
    assert c.w.status == code
    assert c.chain() == before, "a refused call changed the walker's chain"


def test_noalloc_refuses_orphan_transition_row(S, emu):
    c = Caller(S, emu, square(S))
    assert c.call() == 0
    before = c.chain()
    extend_tables_with_orphan_row(c.arrays)
    assert c.call() == ARG and c.chain() == before


@pytest.mark.parametrize("case", ["warmup_L_past_capacity", "ready_L_past_capacity", "ready_n_past_L",
                                  "ready_bad_state", "ready_bad_operator_bond", "ready_bad_operator_vertex",
                                  "phase_3", "phase_negative", "T_zero", "T_nan", "ready_num_worms_huge",
                                  "ready_num_worms_inf", "ready_avg_worm_length_negative",
                                  "new_init_num_worms_inf"])
def test_noalloc_refuses_bad_walker(S, emu, case):
    flat = square(S)
    c = Caller(S, emu, flat)
    assert c.call() == 0
    w = c.w
    if case == "warmup_L_past_capacity":
        w.phase, w.warmup_done, w.L = 1, 1, len(c.ops) + 1
    elif case == "ready_L_past_capacity":
        w.L = len(c.ops) + 1
    elif case == "ready_n_past_L":
        w.num_operators = w.L + 1
    elif case == "ready_bad_state":
        c.state[3] = 2
    elif case == "ready_bad_operator_bond":
        c.ops[0] = 1 | (3 << 1) | (flat.nbonds << 11)
    elif case == "ready_bad_operator_vertex":
        c.ops[0] = 1 | (2 * 6 + 1) << 1
    elif case == "phase_3":
        w.phase = 3
    elif case == "phase_negative":
        w.phase = -1
    elif case == "T_zero":
        w.T = 0.0
    elif case == "T_nan":
        w.T = float("nan")
    elif case == "ready_num_worms_huge":  # a sweep runs ceil(num_worms) worms
        w.num_worms = 2.0 ** 40
    elif case == "ready_num_worms_inf":
        w.num_worms = float("inf")
    elif case == "ready_avg_worm_length_negative":
        w.avg_worm_length = -1.0
    elif case == "new_init_num_worms_inf":
        w.phase = 0
        w.init_num_worms = float("inf")
    before = c.chain()
    assert c.call() == ARG, case
    assert c.chain() == before


def test_noalloc_warmup_walker_resumes(S, O, emu):
    """A walker left in its diagonal warm-up (phase 1) by a capacity stop is checked like an
    initialised one and, with a valid opstring, resumes to the oracle's chain."""
    flat = square(S, 8)
    c = Caller(S, emu, flat, cap=64)
    rc = c.call(nsweeps=3)
    assert rc == 3 and c.w.phase == 1  # SSE_ERR_CAPACITY during Carlo.init!'s warm-up sweeps
    bigger = np.zeros(c.w.need_capacity + 64, dtype=np.uint32)
    bigger[: c.w.L] = c.ops[: c.w.L]
    c.ops = bigger
    while True:
        rc = c.call(nsweeps=3 - (c.w.sweeps if c.w.phase == 2 else 0))
        if rc != 3:
            break
        bigger = np.zeros(c.w.need_capacity + 64, dtype=np.uint32)
        bigger[: c.w.L] = c.ops[: c.w.L]
        c.ops = bigger
    assert rc == 0 and c.w.sweeps == 3
    o = O.OracleWalker(O.OracleModel(flat), T=0.5, seed=7, stream=3, thermalization=1)
    o.init()
    o.run(3, measure=True)
    assert c.w.L == o.w.L and c.w.rng_counter == o.w.ctr
    assert np.array_equal(c.ops[: c.w.L], o.ops) and np.array_equal(c.state, o.state)


def test_host_registration_refuses_the_same_tables(S, fake):
    """sse_model_register refuses the table corruptions above that it can see (all but the
    over-long row, which it reports as SSE_ERR_UNSUPPORTED), and the orphan row."""
    from sse_gb300.engine import Engine, SSEError

    eng = Engine(0, library=fake)
    try:
        flat = square(S)
        for name, corrupt, code in TABLE_CASES + [("orphan row", extend_tables_with_orphan_row, ARG)]:
            c = Caller(S, fake, flat)
            corrupt(c.arrays)

            class F:
                pass

            f = F()
            for k in ("nsites", "nbonds", "ntypes", "maxdim", "nest", "energy_offset", "norm_site_count"):
                setattr(f, k, getattr(flat, k))
            f.arrays = c.arrays
            with pytest.raises(SSEError) as err:
                eng.register_model(f)
            assert err.value.code == code, name
    finally:
        eng.close()
