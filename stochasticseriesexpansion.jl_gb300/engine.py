"""ctypes binding of the C ABI in include/sse_gpu.h.

This is the only path to the GPU engine: it loads the in-tree
``_build/libssegpu.so`` and raises if the library is missing.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB

# SSE_GPU_ABI_VERSION of include/sse_gpu.h whose structs these bindings mirror
ABI_VERSION = 3

P = C.POINTER

SSE_SWEEP_MEASURE = 1
SSE_SWEEP_PLAIN = 2
SSE_SWEEP_GRAPH = 4

STATUS_NAMES = {
    0: "SSE_OK", 1: "SSE_ERR_ARG", 2: "SSE_ERR_CUDA", 3: "SSE_ERR_CAPACITY", 4: "SSE_ERR_INVALID_VERTEX",
    5: "SSE_ERR_TIMEOUT", 6: "SSE_ERR_NOMEM", 7: "SSE_ERR_STATE", 8: "SSE_ERR_WORM_CAP", 9: "SSE_ERR_UNSUPPORTED",
}

OBS_BASE_NAMES = ["Sign", "OperatorCount", "SignOperatorCount", "SignOperatorCount2", "SignEnergy", "WormLengthFraction"]
OBS_EST_NAMES = ["SignMag", "SignAbsMag", "SignMag2", "SignMag4", "SignMagChi"]


def observable_names(est_prefixes):
    names = list(OBS_BASE_NAMES)
    for p in est_prefixes:
        names += [n.replace("Sign", "Sign" + p, 1) for n in OBS_EST_NAMES]
    return names


class SSEError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class ModelDesc(C.Structure):
    _fields_ = [
        ("nsites", C.c_int32), ("nbonds", C.c_int32), ("ntypes", C.c_int32), ("maxdim", C.c_int32), ("nest", C.c_int32),
        ("energy_offset", C.c_double), ("norm_site_count", C.c_double),
        ("site_dims", P(C.c_int32)), ("bond_type", P(C.c_int32)), ("bond_sites", P(C.c_int32)),
        ("type_dims", P(C.c_int32)), ("type_nverts", P(C.c_int32)), ("type_maxworm", P(C.c_int32)),
        ("type_diag_off", P(C.c_int32)), ("type_vert_off", P(C.c_int32)), ("type_trans_off", P(C.c_int32)),
        ("diag_vertex", P(C.c_int32)), ("weight", P(C.c_double)), ("sign", P(C.c_int8)), ("leg_state", P(C.c_uint8)),
        ("trans_start", P(C.c_int32)), ("trans_count", P(C.c_int32)), ("out_cum", P(C.c_double)),
        ("out_target", P(C.c_int32)), ("out_leg", P(C.c_int8)), ("out_worm", P(C.c_int8)), ("est_coef", P(C.c_double)),
    ]


class WalkerParams(C.Structure):
    _fields_ = [
        ("T", C.c_double), ("seed", C.c_uint64), ("stream", C.c_uint64), ("init_opstring_cutoff", C.c_int64),
        ("diagonal_warmup_sweeps", C.c_int32), ("init_num_worms", C.c_double),
        ("num_worms_attenuation_factor", C.c_double), ("target_worm_length_fraction", C.c_double),
        ("thermalization", C.c_int64),
    ]


class WalkerInfo(C.Structure):
    _fields_ = [
        ("L", C.c_int64), ("num_operators", C.c_int64), ("capacity", C.c_int64), ("sweeps", C.c_int64),
        ("rng_counter", C.c_uint64), ("num_worms", C.c_double), ("avg_worm_length", C.c_double), ("T", C.c_double),
        ("status", C.c_int32), ("model", C.c_int32), ("resize_after_thermalization", C.c_int64),
        ("slot_visits", C.c_int64), ("worm_steps", C.c_int64), ("phase_cycles", C.c_int64 * 4),
        ("worm_undos", C.c_int64),
    ]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["phase_cycles"] = list(self.phase_cycles)
        return d


class NoAllocWalker(C.Structure):
    """sse_noalloc_walker: one walker kept by the caller in device memory."""

    _fields_ = [
        ("T", C.c_double), ("seed", C.c_uint64), ("stream", C.c_uint64), ("init_opstring_cutoff", C.c_int64),
        ("diagonal_warmup_sweeps", C.c_int32), ("phase", C.c_int32), ("init_num_worms", C.c_double),
        ("num_worms_attenuation_factor", C.c_double), ("target_worm_length_fraction", C.c_double),
        ("thermalization", C.c_int64), ("L", C.c_int64), ("num_operators", C.c_int64), ("sweeps", C.c_int64),
        ("rng_counter", C.c_uint64), ("num_worms", C.c_double), ("avg_worm_length", C.c_double),
        ("warmup_done", C.c_int32), ("status", C.c_int32), ("need_capacity", C.c_int64),
        ("slot_visits", C.c_int64), ("worm_steps", C.c_int64), ("worm_undos", C.c_int64),
    ]


_lib = None


def lib():
    """The engine library (libssegpu.so, built for sm_103a), loaded once."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} is not built: run __graft_entry__.build() (nvcc, sm_103a)")
        _lib = load_library(LIB)
    return _lib


def load_library(path: str):
    """Loads a build of the engine library from `path` and declares the C ABI's signatures on it."""
    L = C.CDLL(path)
    I32, I64, U32 = C.c_int32, C.c_int64, C.c_uint32
    eng = C.c_void_p
    sig = {
        "sse_abi_version": ([], C.c_int),
        "sse_engine_create": ([I32, P(eng)], C.c_int),
        "sse_engine_destroy": ([eng], C.c_int),
        "sse_engine_last_error": ([eng], C.c_char_p),
        "sse_model_register": ([eng, P(ModelDesc), P(I32)], C.c_int),
        "sse_model_nobs": ([eng, I32, P(I32)], C.c_int),
        "sse_walkers_create": ([eng, I32, I32, P(WalkerParams), P(I32)], C.c_int),
        "sse_walkers_destroy": ([eng, I32, P(I32)], C.c_int),
        "sse_walkers_reserve": ([eng, I32, P(I32), I64], C.c_int),
        "sse_walkers_init": ([eng, I32, P(I32)], C.c_int),
        "sse_sweep": ([eng, I32, P(I32), I32, U32], C.c_int),
        "sse_sweep_each": ([eng, I32, P(I32), P(I32), U32], C.c_int),
        "sse_observables": ([eng, I32, P(I32), P(C.c_double), P(I64), P(C.c_double), I32], C.c_int),
        "sse_walker_info_get": ([eng, I32, P(WalkerInfo)], C.c_int),
        "sse_walker_export": ([eng, I32, P(U32), I64, P(C.c_uint8), P(WalkerInfo)], C.c_int),
        "sse_walker_import": ([eng, I32, P(U32), P(C.c_uint8), P(WalkerInfo)], C.c_int),
        "sse_vertex_list": ([eng, I32, P(I32), P(I32), P(I32)], C.c_int),
        "sse_last_timing": ([eng, P(C.c_double), P(I64)], C.c_int),
        "sse_set_launch": ([eng, I32, I32], C.c_int),
        "sse_get_launch": ([eng, P(I32), P(I32)], C.c_int),
        "sse_profiler_range": ([eng, I32], C.c_int),
        "sse_autotune": ([eng, I32, P(I32), I32, U32, P(I32), P(I32), P(C.c_double)], C.c_int),
        "sse_autotune_each": ([eng, I32, P(I32), P(I32), U32, P(I32), P(I32), P(C.c_double)], C.c_int),
        "sse_set_staging": ([eng, I32], C.c_int),
        "sse_get_staging": ([eng, P(I32)], C.c_int),
        "sse_walker_set_T": ([eng, I32, C.c_double], C.c_int),
        "sse_walkers_set_worm_cap": ([eng, I32, P(I32), I32], C.c_int),
        "sse_check_walkers": ([eng, I32, P(I32), P(I32)], C.c_int),
        "sse_tempering_exchange": ([eng, I32, I32, P(I32), C.c_uint64, C.c_uint64, P(I32)], C.c_int),
        "sse_sweep_tempering": ([eng, I32, I32, P(I32), I32, I32, C.c_uint64, C.c_uint64, U32, P(I64), P(I64)],
                                C.c_int),
        "sse_sweep_noalloc": ([P(ModelDesc), C.c_void_p, C.c_void_p, I64, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, I32, U32], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    if L.sse_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{path} has ABI version {L.sse_abi_version()}, these bindings mirror version "
                           f"{ABI_VERSION}: rebuild it with __graft_entry__.build()")
    return L


def exported_symbols():
    """Names of the C ABI entry points this binding expects the library to export."""
    return [
        "sse_abi_version", "sse_engine_create", "sse_engine_destroy", "sse_engine_last_error", "sse_model_register",
        "sse_model_nobs", "sse_walkers_create", "sse_walkers_destroy", "sse_walkers_reserve", "sse_walkers_init",
        "sse_sweep", "sse_sweep_each", "sse_observables", "sse_walker_info_get", "sse_walker_export", "sse_walker_import",
        "sse_vertex_list", "sse_last_timing", "sse_set_launch", "sse_get_launch", "sse_profiler_range", "sse_autotune",
        "sse_sweep_noalloc", "sse_walker_set_T", "sse_tempering_exchange", "sse_sweep_tempering",
        "sse_set_staging", "sse_get_staging", "sse_autotune_each", "sse_walkers_set_worm_cap",
        "sse_check_walkers",
    ]


def device_model_desc(flat, device_ptr):
    """An sse_model_desc whose array pointers are device addresses: ``device_ptr(name, array)``
    returns the device address holding a copy of ``flat.arrays[name]`` (the caller owns that memory)."""
    a = flat.arrays
    q = lambda name, t: C.cast(C.c_void_p(device_ptr(name, a[name])), P(t))  # noqa: E731
    return ModelDesc(
        flat.nsites, flat.nbonds, flat.ntypes, flat.maxdim, flat.nest, flat.energy_offset, flat.norm_site_count,
        q("site_dims", C.c_int32), q("bond_type", C.c_int32), q("bond_sites", C.c_int32), q("type_dims", C.c_int32),
        q("type_nverts", C.c_int32), q("type_maxworm", C.c_int32), q("type_diag_off", C.c_int32),
        q("type_vert_off", C.c_int32), q("type_trans_off", C.c_int32), q("diag_vertex", C.c_int32),
        q("weight", C.c_double), q("sign", C.c_int8), q("leg_state", C.c_uint8), q("trans_start", C.c_int32),
        q("trans_count", C.c_int32), q("out_cum", C.c_double), q("out_target", C.c_int32), q("out_leg", C.c_int8),
        q("out_worm", C.c_int8), q("est_coef", C.c_double),
    )


def sweep_noalloc(desc, walker, ops, ops_capacity, state, obs_sum, obs_count, obs_last, nsweeps, flags=SSE_SWEEP_MEASURE):
    """sse_sweep_noalloc with device addresses (ints) for every buffer; returns the sse_status."""
    return lib().sse_sweep_noalloc(C.byref(desc), C.c_void_p(walker), C.c_void_p(ops), int(ops_capacity),
                                   C.c_void_p(state), C.c_void_p(obs_sum), C.c_void_p(obs_count),
                                   C.c_void_p(obs_last), int(nsweeps), int(flags))


def _p(a, t):
    return a.ctypes.data_as(P(t))


# the flat model tables in sse_model_desc order, with their C element types
MODEL_TABLES = (
    ("site_dims", np.int32), ("bond_type", np.int32), ("bond_sites", np.int32), ("type_dims", np.int32),
    ("type_nverts", np.int32), ("type_maxworm", np.int32), ("type_diag_off", np.int32), ("type_vert_off", np.int32),
    ("type_trans_off", np.int32), ("diag_vertex", np.int32), ("weight", np.float64), ("sign", np.int8),
    ("leg_state", np.uint8), ("trans_start", np.int32), ("trans_count", np.int32), ("out_cum", np.float64),
    ("out_target", np.int32), ("out_leg", np.int8), ("out_worm", np.int8), ("est_coef", np.float64),
)
_CTYPE = {np.int32: C.c_int32, np.float64: C.c_double, np.int8: C.c_int8, np.uint8: C.c_uint8}


def model_table(arrays, name, dtype):
    """arrays[name] as a C-contiguous array of the table's C element type; a conversion that would
    change a value (overflow, a fraction in an integer table) raises ValueError."""
    x = np.asarray(arrays[name])
    y = np.ascontiguousarray(x.reshape(-1), dtype=dtype)
    if x.dtype != y.dtype and not np.array_equal(y, x.reshape(-1)):
        raise ValueError(f"model table {name!r}: values do not fit {np.dtype(dtype).name}")
    return y


def _ids(ids):
    a = np.ascontiguousarray(ids, dtype=np.int32)
    return a, _p(a, C.c_int32)


class Engine:
    """One GPU, one stream, many walkers (see include/sse_gpu.h)."""

    def __init__(self, device: int = 0, library=None):
        """`library`: a handle from load_library (default: the sm_103a build)."""
        self._L = library if library is not None else lib()
        self.h = C.c_void_p()
        rc = self._L.sse_engine_create(device, C.byref(self.h))
        if rc != 0:
            raise SSEError(rc, "sse_engine_create failed")
        self._models = {}
        self._walker_model = {}

    def close(self):
        if self.h:
            self._L.sse_engine_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise SSEError(rc, (self._L.sse_engine_last_error(self.h) or b"").decode())

    # ---- models ----
    def register_model(self, flat) -> int:
        # converted copies stay referenced here until the library has copied them to the device
        tables = [model_table(flat.arrays, name, dt) for name, dt in MODEL_TABLES]
        d = ModelDesc(
            flat.nsites, flat.nbonds, flat.ntypes, flat.maxdim, flat.nest, flat.energy_offset, flat.norm_site_count,
            *[_p(t, _CTYPE[dt]) for t, (_, dt) in zip(tables, MODEL_TABLES)],
        )
        mid = C.c_int32()
        self._check(self._L.sse_model_register(self.h, C.byref(d), C.byref(mid)))
        del tables
        self._models[mid.value] = flat
        return mid.value

    def nobs(self, model_id: int) -> int:
        n = C.c_int32()
        self._check(self._L.sse_model_nobs(self.h, model_id, C.byref(n)))
        return n.value

    # ---- walkers ----
    def create_walkers(self, model_id: int, params: list) -> np.ndarray:
        arr = (WalkerParams * len(params))()
        for i, p in enumerate(params):
            arr[i] = WalkerParams(
                float(p["T"]), int(p.get("seed", 0)), int(p.get("stream", i)), int(p.get("init_opstring_cutoff", -1)),
                int(p.get("diagonal_warmup_sweeps", 5)), float(p.get("init_num_worms", 5.0)),
                float(p.get("num_worms_attenuation_factor", 0.01)), float(p.get("target_worm_length_fraction", 2.0)),
                int(p.get("thermalization", 0)),
            )
        ids = np.zeros(len(params), dtype=np.int32)
        self._check(self._L.sse_walkers_create(self.h, model_id, len(params), arr, _p(ids, C.c_int32)))
        for i in ids.tolist():
            self._walker_model[i] = model_id
        return ids

    def destroy_walkers(self, ids):
        a, p = _ids(ids)
        self._check(self._L.sse_walkers_destroy(self.h, len(a), p))
        for i in a.tolist():
            self._walker_model.pop(i, None)

    def reserve(self, ids, capacity: int):
        a, p = _ids(ids)
        self._check(self._L.sse_walkers_reserve(self.h, len(a), p, int(capacity)))

    def init(self, ids):
        a, p = _ids(ids)
        self._check(self._L.sse_walkers_init(self.h, len(a), p))

    def sweep(self, ids, nsweeps: int, measure: bool = True, plain: bool = False, graph: bool = False):
        a, p = _ids(ids)
        flags = (SSE_SWEEP_MEASURE if measure else 0) | (SSE_SWEEP_PLAIN if plain else 0) | (SSE_SWEEP_GRAPH if graph else 0)
        self._check(self._L.sse_sweep(self.h, len(a), p, int(nsweeps), flags))

    def sweep_each(self, ids, nsweeps, measure: bool = True):
        """Per-walker sweep counts in one persistent launch (sse_sweep_each)."""
        a, p = _ids(ids)
        ns = np.ascontiguousarray(nsweeps, dtype=np.int32)
        if len(ns) != len(a):
            raise ValueError("one sweep count per walker")
        self._check(self._L.sse_sweep_each(self.h, len(a), p, _p(ns, C.c_int32), SSE_SWEEP_MEASURE if measure else 0))

    def observables(self, ids, reset: bool = False):
        a, p = _ids(ids)
        nobs = [self.nobs(self._walker_model[i]) for i in a.tolist()]
        tot = int(sum(nobs))
        s = np.zeros(tot)
        c = np.zeros(tot, dtype=np.int64)
        last = np.zeros(tot)
        if len(a):
            self._check(self._L.sse_observables(self.h, len(a), p, _p(s, C.c_double), _p(c, C.c_int64),
                                                _p(last, C.c_double), int(reset)))
        out = []
        o = 0
        for n in nobs:
            out.append((s[o:o + n], c[o:o + n], last[o:o + n]))
            o += n
        return out

    def info(self, wid: int) -> dict:
        inf = WalkerInfo()
        self._check(self._L.sse_walker_info_get(self.h, int(wid), C.byref(inf)))
        return inf.as_dict()

    def export(self, wid: int):
        inf = WalkerInfo()
        self._check(self._L.sse_walker_info_get(self.h, int(wid), C.byref(inf)))
        flat = self._models[self._walker_model[int(wid)]]
        ops = np.zeros(max(inf.L, 1), dtype=np.uint32)
        st = np.zeros(flat.nsites, dtype=np.uint8)
        self._check(self._L.sse_walker_export(self.h, int(wid), _p(ops, C.c_uint32), len(ops), _p(st, C.c_uint8), C.byref(inf)))
        return ops[: inf.L].copy(), st, inf.as_dict()

    def import_(self, wid: int, ops, state, info: dict):
        ops = np.ascontiguousarray(ops, dtype=np.uint32)
        st = np.ascontiguousarray(state, dtype=np.uint8)
        inf = WalkerInfo()
        for k, _ in WalkerInfo._fields_:
            if k in info and k != "phase_cycles":
                setattr(inf, k, info[k])
        inf.L = len(ops)
        self._check(self._L.sse_walker_import(self.h, int(wid), _p(ops, C.c_uint32) if len(ops) else None,
                                              _p(st, C.c_uint8), C.byref(inf)))

    def vertex_list(self, wid: int):
        inf = self.info(wid)
        flat = self._models[self._walker_model[int(wid)]]
        v = np.zeros(4 * max(inf["L"], 1), dtype=np.int32)
        vf = np.zeros(flat.nsites, dtype=np.int32)
        vl = np.zeros(flat.nsites, dtype=np.int32)
        self._check(self._L.sse_vertex_list(self.h, int(wid), _p(v, C.c_int32), _p(vf, C.c_int32), _p(vl, C.c_int32)))
        return v[: 4 * inf["L"]], vf, vl

    def last_timing(self):
        ms = C.c_double()
        n = C.c_int64()
        self._check(self._L.sse_last_timing(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def autotune(self, ids, nsweeps_probe: int = 5, measure: bool = False):
        """Pick the fastest walkers-per-block and shared-memory staging budget for these walkers (the
        probe sweeps are real Carlo steps); returns (walkers per block, staging bytes, probe ms)."""
        a, p = _ids(ids)
        best = C.c_int32()
        stage = C.c_int32()
        ms = C.c_double()
        self._check(self._L.sse_autotune(self.h, len(a), p, int(nsweeps_probe), SSE_SWEEP_MEASURE if measure else 0,
                                         C.byref(best), C.byref(stage), C.byref(ms)))
        return best.value, stage.value, ms.value

    def autotune_each(self, ids, nsweeps, measure: bool = False):
        """As autotune, each probe giving walker i nsweeps[i] Carlo steps (cost-balanced blocks)."""
        a, p = _ids(ids)
        ns = np.ascontiguousarray(nsweeps, dtype=np.int32)
        if len(ns) != len(a):
            raise ValueError("one sweep count per walker")
        best = C.c_int32()
        stage = C.c_int32()
        ms = C.c_double()
        self._check(self._L.sse_autotune_each(self.h, len(a), p, _p(ns, C.c_int32),
                                              SSE_SWEEP_MEASURE if measure else 0, C.byref(best), C.byref(stage),
                                              C.byref(ms)))
        return best.value, stage.value, ms.value

    def set_staging(self, stage_bytes: int):
        """Shared-memory budget per walker for staging the worm update's records (0: off)."""
        self._check(self._L.sse_set_staging(self.h, int(stage_bytes)))

    def get_staging(self) -> int:
        v = C.c_int32()
        self._check(self._L.sse_get_staging(self.h, C.byref(v)))
        return v.value

    def profiler_range(self, start: bool):
        self._check(self._L.sse_profiler_range(self.h, int(bool(start))))

    def check(self, ids) -> np.ndarray:
        """The reference's isconsistent invariant (plus periodicity, ranges and operator count) on the
        device for every walker: 0 where consistent, else the failing check's code."""
        a, p = _ids(ids)
        out = np.zeros(len(a), dtype=np.int32)
        if len(a):
            self._check(self._L.sse_check_walkers(self.h, len(a), p, _p(out, C.c_int32)))
        return out

    def set_worm_cap(self, ids, factor: int):
        """Worm step cap factor (default 64): a worm longer than factor * max(L + 16, 65536) steps undoes
        its thermalisation sweep's worm phase, or stops the walker in a measured sweep."""
        a, p = _ids(ids)
        self._check(self._L.sse_walkers_set_worm_cap(self.h, len(a), p, int(factor)))

    def set_T(self, wid: int, T: float):
        """Carlo.parallel_tempering_change_parameter!(mc, :T, T) (src/sse.jl:399-405)."""
        self._check(self._L.sse_walker_set_T(self.h, int(wid), float(T)))

    @staticmethod
    def _ladders(ids):
        a = np.ascontiguousarray(ids, dtype=np.int32)
        if a.ndim != 2 or a.shape[1] < 2:
            raise ValueError("ladders are given as an array of shape (nladders, nrungs >= 2)")
        return a, a.shape[0], a.shape[1]

    def tempering_exchange(self, ladders, seed: int, step: int) -> np.ndarray:
        """One parallel-tempering exchange step (sse_tempering_exchange); returns the accept flags
        (1, 0, or -1 for pairs not proposed), shape (nladders, nrungs - 1), pairs in T order."""
        a, nl, nr = self._ladders(ladders)
        acc = np.zeros((nl, nr - 1), dtype=np.int32)
        self._check(self._L.sse_tempering_exchange(self.h, nl, nr, _p(a, C.c_int32), int(seed), int(step),
                                                   _p(acc, C.c_int32)))
        return acc

    def sweep_tempering(self, ladders, nblocks: int, interval: int, seed: int, first_step: int = 0,
                        measure: bool = True, graph: bool = False):
        """nblocks x (interval Carlo steps + one exchange step); returns (accepted, proposed) counts per
        rung pair, shape (nladders, nrungs - 1)."""
        a, nl, nr = self._ladders(ladders)
        acc = np.zeros((nl, nr - 1), dtype=np.int64)
        prop = np.zeros((nl, nr - 1), dtype=np.int64)
        flags = (SSE_SWEEP_MEASURE if measure else 0) | (SSE_SWEEP_GRAPH if graph else 0)
        self._check(self._L.sse_sweep_tempering(self.h, nl, nr, _p(a, C.c_int32), int(nblocks), int(interval),
                                                int(seed), int(first_step), flags, _p(acc, C.c_int64),
                                                _p(prop, C.c_int64)))
        return acc, prop

    def set_launch(self, warps_per_block: int = 0, blocks_per_sm: int = 0):
        """Warps (walkers) per block of the batched kernel (1..4; 0 = automatic) and a cap on blocks per SM."""
        self._check(self._L.sse_set_launch(self.h, warps_per_block, blocks_per_sm))
