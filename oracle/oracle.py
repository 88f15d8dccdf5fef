"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Used by ``tests/``, ``__graft_entry__.smoke()`` and the benchmark's CPU
baseline, to check results and to time the CPU path.  The GPU engine never
imports this module.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsse_oracle.so")

ORC_OBS_BASE = 6
ORC_OBS_PER_EST = 5
OBS_BASE_NAMES = ["Sign", "OperatorCount", "SignOperatorCount", "SignOperatorCount2", "SignEnergy", "WormLengthFraction"]
OBS_EST_NAMES = ["SignMag", "SignAbsMag", "SignMag2", "SignMag4", "SignMagChi"]


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
        os.path.getmtime(os.path.join(HERE, f)) for f in ("sse_oracle.c", "sse_oracle.h")
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


P = C.POINTER


class OrcModel(C.Structure):
    _fields_ = [
        ("nsites", C.c_int32),
        ("nbonds", C.c_int32),
        ("ntypes", C.c_int32),
        ("maxdim", C.c_int32),
        ("nest", C.c_int32),
        ("energy_offset", C.c_double),
        ("norm_site_count", C.c_double),
        ("site_dims", P(C.c_int32)),
        ("bond_type", P(C.c_int32)),
        ("bond_sites", P(C.c_int32)),
        ("type_dims", P(C.c_int32)),
        ("type_nverts", P(C.c_int32)),
        ("type_maxworm", P(C.c_int32)),
        ("type_diag_off", P(C.c_int32)),
        ("type_vert_off", P(C.c_int32)),
        ("type_trans_off", P(C.c_int32)),
        ("diag_vertex", P(C.c_int32)),
        ("weight", P(C.c_double)),
        ("sign", P(C.c_int8)),
        ("leg_state", P(C.c_uint8)),
        ("trans_start", P(C.c_int32)),
        ("trans_count", P(C.c_int32)),
        ("out_cum", P(C.c_double)),
        ("out_target", P(C.c_int32)),
        ("out_leg", P(C.c_int8)),
        ("out_worm", P(C.c_int8)),
        ("est_coef", P(C.c_double)),
    ]


class OrcWalker(C.Structure):
    _fields_ = [
        ("T", C.c_double),
        ("target_worm_length_fraction", C.c_double),
        ("num_worms_attenuation_factor", C.c_double),
        ("seed", C.c_uint64),
        ("stream", C.c_uint64),
        ("thermalization", C.c_int64),
        ("avg_worm_length", C.c_double),
        ("num_worms", C.c_double),
        ("num_operators", C.c_int64),
        ("L", C.c_int64),
        ("ctr", C.c_uint64),
        ("sweeps", C.c_int64),
        ("ops", P(C.c_uint32)),
        ("ops_cap", C.c_int64),
        ("state", P(C.c_uint8)),
        ("vertices", P(C.c_int32)),
        ("vertices_len", C.c_int64),
        ("v_first", P(C.c_int32)),
        ("v_last", P(C.c_int32)),
        ("status", C.c_int32),
        ("resize_after_thermalization", C.c_int64),
        ("worm_steps_total", C.c_int64),
        ("slot_visits_total", C.c_int64),
        ("nobs", C.c_int32),
        ("obs_sum", P(C.c_double)),
        ("obs_last", P(C.c_double)),
        ("obs_count", P(C.c_int64)),
        ("worm_cap_factor", C.c_int32),
        ("worm_undos", C.c_int64),
        ("ops_saved", P(C.c_uint32)),
        ("ops_saved_cap", C.c_int64),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.orc_walker_create.restype = P(OrcWalker)
        L.orc_walker_create.argtypes = [P(OrcModel), C.c_double, C.c_uint64, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_int64]
        L.orc_walker_destroy.argtypes = [P(OrcWalker)]
        L.orc_init.argtypes = [P(OrcModel), P(OrcWalker), C.c_int64, C.c_int32]
        L.orc_sweep.argtypes = [P(OrcModel), P(OrcWalker), C.c_int32]
        L.orc_measure.argtypes = [P(OrcModel), P(OrcWalker)]
        L.orc_step.argtypes = [P(OrcModel), P(OrcWalker), C.c_int32]
        L.orc_run.argtypes = [P(OrcModel), P(OrcWalker), C.c_int64, C.c_int32]
        L.orc_diagonal_update.argtypes = [P(OrcModel), P(OrcWalker), C.c_int32]
        L.orc_make_vertex_list.argtypes = [P(OrcModel), P(OrcWalker)]
        L.orc_worm_update.argtypes = [P(OrcModel), P(OrcWalker), C.c_int32]
        L.orc_set_opstring.argtypes = [P(OrcWalker), P(C.c_uint32), C.c_int64, C.c_int64]
        L.orc_set_state.argtypes = [P(OrcModel), P(OrcWalker), P(C.c_uint8)]
        L.orc_run_parallel.argtypes = [P(OrcModel), P(P(OrcWalker)), C.c_int32, C.c_int64, C.c_int32, C.c_int32]
        L.orc_philox4x32_10.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
        L.orc_draw.restype = C.c_uint64
        L.orc_draw.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.orc_tanh.restype = C.c_double
        L.orc_tanh.argtypes = [C.c_double]
        L.orc_tempering_weight.restype = C.c_double
        L.orc_tempering_weight.argtypes = [C.c_double, C.c_double, C.c_int64, C.c_int64]
        L.orc_tempering_exchange.restype = C.c_int
        L.orc_tempering_exchange.argtypes = [P(P(OrcWalker)), C.c_int32, C.c_int32, C.c_uint64, C.c_uint64, P(C.c_int32)]
        for f in ("orc_init", "orc_sweep", "orc_measure", "orc_step", "orc_run", "orc_diagonal_update",
                  "orc_make_vertex_list", "orc_worm_update", "orc_set_opstring", "orc_set_state", "orc_run_parallel"):
            getattr(L, f).restype = C.c_int
    return _lib


def _ptr(a, ctype):
    return a.ctypes.data_as(P(ctype))


class OracleModel:
    """Holds the flat arrays of a ``FlatModel`` alive and exposes an ``OrcModel``."""

    def __init__(self, flat):
        self.flat = flat
        a = flat.arrays
        self._keep = a
        self.s = OrcModel(
            flat.nsites, flat.nbonds, flat.ntypes, flat.maxdim, flat.nest, flat.energy_offset, flat.norm_site_count,
            _ptr(a["site_dims"], C.c_int32), _ptr(a["bond_type"], C.c_int32), _ptr(a["bond_sites"], C.c_int32),
            _ptr(a["type_dims"], C.c_int32), _ptr(a["type_nverts"], C.c_int32), _ptr(a["type_maxworm"], C.c_int32),
            _ptr(a["type_diag_off"], C.c_int32), _ptr(a["type_vert_off"], C.c_int32), _ptr(a["type_trans_off"], C.c_int32),
            _ptr(a["diag_vertex"], C.c_int32), _ptr(a["weight"], C.c_double), _ptr(a["sign"], C.c_int8),
            _ptr(a["leg_state"], C.c_uint8), _ptr(a["trans_start"], C.c_int32), _ptr(a["trans_count"], C.c_int32),
            _ptr(a["out_cum"], C.c_double), _ptr(a["out_target"], C.c_int32), _ptr(a["out_leg"], C.c_int8),
            _ptr(a["out_worm"], C.c_int8),
            _ptr(a["est_coef"], C.c_double) if len(a["est_coef"]) else None,
        )
        self.ref = C.byref(self.s)


class OracleWalker:
    def __init__(self, model: OracleModel, T, seed, stream, init_num_worms=5.0, attenuation=0.01,
                 target_fraction=2.0, thermalization=0):
        self.model = model
        self.p = lib().orc_walker_create(model.ref, T, seed, stream, init_num_worms, attenuation, target_fraction, thermalization)
        if not self.p:
            raise MemoryError("orc_walker_create failed")
        self.w = self.p.contents

    def __del__(self):
        p = getattr(self, "p", None)
        if p and _lib is not None:
            _lib.orc_walker_destroy(p)
            self.p = None

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"oracle error {rc} (status {self.w.status})")

    def init(self, init_cutoff=-1, warmup=5):
        self._check(lib().orc_init(self.model.ref, self.p, init_cutoff, warmup))

    def sweep(self, thermalized=False):
        self._check(lib().orc_sweep(self.model.ref, self.p, int(thermalized)))

    def measure(self):
        self._check(lib().orc_measure(self.model.ref, self.p))

    def step(self, measure=True):
        self._check(lib().orc_step(self.model.ref, self.p, int(measure)))

    def run(self, nsteps, measure=True):
        self._check(lib().orc_run(self.model.ref, self.p, nsteps, int(measure)))

    def diagonal_update(self, thermalized=False):
        self._check(lib().orc_diagonal_update(self.model.ref, self.p, int(thermalized)))

    def make_vertex_list(self):
        self._check(lib().orc_make_vertex_list(self.model.ref, self.p))

    def worm_update(self, thermalized=False):
        self._check(lib().orc_worm_update(self.model.ref, self.p, int(thermalized)))

    def set_opstring(self, ops, num_operators=None):
        ops = np.ascontiguousarray(ops, dtype=np.uint32)
        if num_operators is None:
            num_operators = int(np.count_nonzero(ops))
        self._check(lib().orc_set_opstring(self.p, _ptr(ops, C.c_uint32), len(ops), num_operators))

    def set_state(self, state):
        st = np.ascontiguousarray(state, dtype=np.uint8)
        self._check(lib().orc_set_state(self.model.ref, self.p, _ptr(st, C.c_uint8)))

    # ---- views ----
    @property
    def ops(self):
        return np.ctypeslib.as_array(self.w.ops, shape=(self.w.L,)).copy() if self.w.L else np.zeros(0, np.uint32)

    @property
    def state(self):
        return np.ctypeslib.as_array(self.w.state, shape=(self.model.flat.nsites,)).copy()

    @property
    def vertices(self):
        n = self.w.vertices_len * 4
        return np.ctypeslib.as_array(self.w.vertices, shape=(n,)).copy() if n else np.zeros(0, np.int32)

    @property
    def v_first(self):
        return np.ctypeslib.as_array(self.w.v_first, shape=(self.model.flat.nsites,)).copy()

    @property
    def v_last(self):
        return np.ctypeslib.as_array(self.w.v_last, shape=(self.model.flat.nsites,)).copy()

    def obs(self):
        n = self.w.nobs
        return (
            np.ctypeslib.as_array(self.w.obs_sum, shape=(n,)).copy(),
            np.ctypeslib.as_array(self.w.obs_count, shape=(n,)).copy(),
            np.ctypeslib.as_array(self.w.obs_last, shape=(n,)).copy(),
        )

    def scalars(self):
        w = self.w
        return dict(L=w.L, n=w.num_operators, ctr=w.ctr, num_worms=w.num_worms, avg_worm_length=w.avg_worm_length,
                    sweeps=w.sweeps, status=w.status)


def run_parallel(model: OracleModel, walkers, nsteps, measure=True, nthreads=1):
    arr = (P(OrcWalker) * len(walkers))(*[w.p for w in walkers])
    rc = lib().orc_run_parallel(model.ref, arr, len(walkers), nsteps, int(measure), nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle error {rc}")


def tempering_exchange(walkers, nladders, nrungs, seed, step):
    """One parallel-tempering exchange step over ladders of oracle walkers (walkers[l*nrungs + k]);
    returns the accept flags per rung pair, shape (nladders, nrungs - 1), and the status."""
    arr = (P(OrcWalker) * len(walkers))(*[w.p for w in walkers])
    acc = np.zeros(nladders * (nrungs - 1), np.int32)
    rc = lib().orc_tempering_exchange(arr, nladders, nrungs, seed, step, _ptr(acc, C.c_int32))
    return acc.reshape(nladders, nrungs - 1), rc


def tempering_weight(Ta, Tb, na, nb):
    return lib().orc_tempering_weight(Ta, Tb, na, nb)


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def draw(seed, stream, index):
    return lib().orc_draw(seed, stream, index)


def tanh(x):
    return lib().orc_tanh(x)
