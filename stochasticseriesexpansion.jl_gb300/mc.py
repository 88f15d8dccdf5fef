"""Python mirror of the reference's Carlo.jl Monte Carlo interface, backed by the GPU engine.

Reference interface (src/sse.jl):

    MC(params)                       src/sse.jl:26-45
    Carlo.init!(mc, ctx, params)     src/sse.jl:47-60
    Carlo.sweep!(mc, ctx)            src/sse.jl:62-68
    Carlo.measure!(mc, ctx)          src/sse.jl:70-87
    Carlo.write_checkpoint / read_checkpoint   src/sse.jl:89-107
    Carlo.register_evaluables        src/sse.jl:111-134, magnetization_estimator.jl:236-258
    Carlo.parallel_tempering_log_weight_ratio / _change_parameter!   src/sse.jl:390-405

``MC`` drives one walker; ``BatchMC`` drives many walkers of one parameter set
in a single persistent launch per sweep block, which is how the engine is
meant to be used; ``TemperingMC`` runs ladders of walkers over a temperature
list with exchange steps on the device.  Both go through ``engine.Engine`` (the C ABI) and raise if
the CUDA library is missing -- there is no CPU fallback.

Parameter names follow the reference: ``T``, ``model`` (a model class such as
``MagnetModel``), ``init_opstring_cutoff``, ``diagonal_warmup_sweeps``,
``init_num_worms``, ``num_worms_attenuation_factor``,
``target_worm_length_fraction``, and the Carlo-level ``thermalization``,
``sweeps``, ``binsize`` and ``seed``.
"""

from __future__ import annotations

import math

import numpy as np

from .engine import Engine, observable_names
from .tables import flatten_model
from .util import dev_to_ref, ref_to_dev


class MCContext:
    """The part of Carlo.MCContext the SSE code uses: the sweep counter, the
    thermalisation rule and the measurement stream (here: per-observable lists)."""

    def __init__(self, params: dict):
        self.thermalization_sweeps = int(params.get("thermalization", 0))
        self.sweeps = 0
        self.seed = int(params.get("seed", 0))
        self.observables: dict = {}

    def is_thermalized(self) -> bool:
        # Carlo: ctx.sweeps > ctx.thermalization_sweeps
        return self.sweeps > self.thermalization_sweeps

    def measure(self, name: str, value: float):
        self.observables.setdefault(name, []).append(float(value))


def _walker_params(params: dict, stream: int) -> dict:
    return dict(
        T=float(params["T"]),
        seed=int(params.get("seed", 0)),
        stream=int(stream),
        init_opstring_cutoff=int(params.get("init_opstring_cutoff", -1)),
        diagonal_warmup_sweeps=int(params.get("diagonal_warmup_sweeps", 5)),
        init_num_worms=float(params.get("init_num_worms", 5)),
        num_worms_attenuation_factor=float(params.get("num_worms_attenuation_factor", 0.01)),
        target_worm_length_fraction=float(params.get("target_worm_length_fraction", 2.0)),
        thermalization=int(params.get("thermalization", 0)),
    )


_ENGINES: dict = {}


def default_engine(device: int = 0) -> Engine:
    if device not in _ENGINES:
        _ENGINES[device] = Engine(device)
    return _ENGINES[device]


class MC:
    """``MC <: AbstractMC`` for one walker (src/sse.jl:6-45)."""

    def __init__(self, params: dict, engine: Engine | None = None, stream: int = 0):
        self.params = params
        self.model = params["model"](params)
        self.flat = flatten_model(self.model)
        self.engine = engine or default_engine(int(params.get("device", 0)))
        self.model_id = self.engine.register_model(self.flat)
        self.wid = int(self.engine.create_walkers(self.model_id, [_walker_params(params, stream)])[0])
        self.names = observable_names(self.flat.est_prefixes)
        self._T = float(params["T"])

    @property
    def T(self) -> float:
        return self._T

    # ---- parallel tempering hooks (src/sse.jl:390-405) ----
    def parallel_tempering_log_weight_ratio(self, parameter: str, new_value: float) -> float:
        if parameter != "T":
            raise ValueError(f"unsupported parallel tempering parameter {parameter}")
        n = self.engine.info(self.wid)["num_operators"]
        return -n * math.log(new_value / self._T)

    def parallel_tempering_change_parameter(self, parameter: str, new_value: float):
        if parameter != "T":
            raise ValueError(f"unsupported parallel tempering parameter {parameter}")
        self.engine.set_T(self.wid, float(new_value))
        self._T = float(new_value)

    # ---- Carlo.AbstractMC ----
    def init(self, ctx: MCContext, params: dict | None = None):
        self.engine.init([self.wid])

    def sweep(self, ctx: MCContext):
        """One Carlo step: sweep!, ctx.sweeps += 1, and the engine's measure! when thermalised."""
        self.engine.sweep([self.wid], 1, measure=True)
        ctx.sweeps += 1

    def measure(self, ctx: MCContext):
        """Forward the observables produced since the last call (one step: one value each) to the context."""
        s, c, _ = self.engine.observables([self.wid], reset=True)[0]
        for i, name in enumerate(self.names):
            if c[i] > 0:
                ctx.measure(name, s[i] / c[i])

    def write_checkpoint(self) -> dict:
        """The reference's checkpoint fields (src/sse.jl:89-97) plus the replay counter;
        opcodes in the reference's UInt64 layout and 1-based states."""
        ops, st, inf = self.engine.export(self.wid)
        return {
            "num_operators": inf["num_operators"],
            "avg_worm_length": inf["avg_worm_length"],
            "num_worms": inf["num_worms"],
            "operators": dev_to_ref(ops),
            "state": st.astype(np.uint8) + 1,
            "rng_counter": inf["rng_counter"],
            "sweeps": inf["sweeps"],
        }

    def read_checkpoint(self, d: dict):
        ops = ref_to_dev(np.asarray(d["operators"], dtype=np.uint64))
        st = np.asarray(d["state"], dtype=np.int64) - 1
        self.engine.import_(self.wid, ops, st.astype(np.uint8), dict(
            num_operators=int(d["num_operators"]), avg_worm_length=float(d["avg_worm_length"]),
            num_worms=float(d["num_worms"]), rng_counter=int(d.get("rng_counter", 0)), sweeps=int(d.get("sweeps", 0))))


def evaluables(means: dict, est_prefixes, norm_sites: float) -> dict:
    """Carlo evaluables (src/sse.jl:124-131, magnetization_estimator.jl:236-258)."""
    out = {}
    s = means["Sign"]
    out["Energy"] = means["SignEnergy"] / s
    out["SpecificHeat"] = (means["SignOperatorCount2"] / s - means["SignOperatorCount"] ** 2 / s**2
                           - means["SignOperatorCount"] / s) / norm_sites
    for p in est_prefixes:
        for n in ("Mag", "AbsMag", "Mag2", "Mag4", "MagChi"):
            out[p + n] = means["Sign" + p + n] / s
        s2, s4 = means["Sign" + p + "Mag2"], means["Sign" + p + "Mag4"]
        out[p + "BinderRatio"] = 0.0 if (s2 == 0 and s4 == 0) else s2**2 / s4 / s
    return out


class BatchMC:
    """Many walkers of one parameter set: ``nwalkers`` chains with streams 0..nwalkers-1."""

    def __init__(self, params: dict, nwalkers: int, engine: Engine | None = None, first_stream: int = 0):
        self.params = params
        self.model = params["model"](params)
        self.flat = flatten_model(self.model)
        self.engine = engine or default_engine(int(params.get("device", 0)))
        self.model_id = self.engine.register_model(self.flat)
        self.ids = self.engine.create_walkers(
            self.model_id, [_walker_params(params, first_stream + k) for k in range(nwalkers)])
        self.names = observable_names(self.flat.est_prefixes)
        self.bins: list = []

    def init(self):
        self.engine.init(self.ids)

    def sweep(self, nsweeps: int, measure: bool = True):
        self.engine.sweep(self.ids, nsweeps, measure=measure)

    def collect_bin(self):
        """Per-walker means of everything measured since the last bin (one bin per walker)."""
        out = self.engine.observables(self.ids, reset=True)
        for s, c, _ in out:
            self.bins.append({n: (s[i] / c[i] if c[i] else np.nan) for i, n in enumerate(self.names)})

    def run(self, sweeps: int, binsize: int):
        """init!, thermalisation, then measured sweeps in bins of `binsize`."""
        therm = int(self.params.get("thermalization", 0))
        self.init()
        done = 0
        while done < therm:
            k = min(binsize, therm - done)
            self.sweep(k)
            done += k
        self.engine.observables(self.ids, reset=True)
        for _ in range(max(1, sweeps // binsize)):
            self.sweep(binsize)
            self.collect_bin()

    def results(self) -> dict:
        """Evaluables with jackknife errors over all bins of all walkers: name -> (mean, error)."""
        return jackknife_results(self.bins, self.names, self.flat)


def jackknife_results(bins: list, names: list, flat) -> dict:
    """Evaluables with jackknife errors over bins (dicts of observable means): name -> (mean, error).

    A bin without measurements (NaN means: a walker that measured nothing in it) is left out, so it
    does not pull the means towards zero; with fewer than two bins the errors are NaN."""
    keys = [k for k in names if not all(np.isnan(b[k]) for b in bins)]
    bins = [b for b in bins if not any(np.isnan(b[k]) for k in keys)]
    nb = len(bins)
    if nb == 0 or not keys:
        return {}
    arr = {k: np.array([b[k] for b in bins]) for k in keys}
    tot = {k: v.sum() for k, v in arr.items()}
    full = evaluables({k: tot[k] / nb for k in keys}, flat.est_prefixes, flat.norm_site_count)
    res = {}
    if nb < 2:
        for name, v in full.items():
            res[name] = (v, float("nan"))
        for k in keys:
            res.setdefault(k, (float(arr[k][0]), float("nan")))
        return res
    loo = [evaluables({k: (tot[k] - arr[k][i]) / (nb - 1) for k in keys}, flat.est_prefixes, flat.norm_site_count)
           for i in range(nb)]
    for name, v in full.items():
        x = np.array([l[name] for l in loo])
        res[name] = (v, float(np.sqrt((nb - 1) / nb * np.sum((x - x.mean()) ** 2))))
    for k in keys:
        res.setdefault(k, (float(arr[k].mean()), float(arr[k].std() / np.sqrt(nb))))
    return res


class TemperingMC:
    """Parallel tempering in T (src/sse.jl:390-405) over resident walkers.

    ``nladders`` independent ladders, each holding one walker per entry of ``temperatures`` (walker
    (l, k) starts at temperatures[k] with stream first_stream + l*len(temperatures) + k).  Every
    ``interval`` Carlo steps the device runs one exchange step: the walkers of a ladder, ranked by
    T, propose the rung pairs (k, k+1) with k of alternating parity and swap temperatures with the
    Metropolis weight built from parallel_tempering_log_weight_ratio.  The observable accumulators
    move with the temperature, so every bin is per temperature.
    """

    def __init__(self, params: dict, temperatures, nladders: int = 1, interval: int = 10,
                 engine: Engine | None = None, first_stream: int = 0, exchange_seed: int | None = None):
        temps = [float(t) for t in temperatures]
        if len(temps) < 2 or len(set(temps)) != len(temps):
            raise ValueError("a ladder needs at least two distinct temperatures")
        self.params = params
        self.temperatures = temps
        self.interval = int(interval)
        self.model = params["model"](params)
        self.flat = flatten_model(self.model)
        self.engine = engine or default_engine(int(params.get("device", 0)))
        self.model_id = self.engine.register_model(self.flat)
        nr = len(temps)
        wp = []
        for l in range(nladders):
            for k in range(nr):
                p = _walker_params(dict(params, T=temps[k]), first_stream + l * nr + k)
                wp.append(p)
        self.ladders = self.engine.create_walkers(self.model_id, wp).reshape(nladders, nr)
        self.names = observable_names(self.flat.est_prefixes)
        self.seed = int(params.get("seed", 0)) if exchange_seed is None else int(exchange_seed)
        self.step = 0
        self.accepted = np.zeros((nladders, nr - 1), dtype=np.int64)
        self.proposed = np.zeros((nladders, nr - 1), dtype=np.int64)
        self.bins: list = [[] for _ in temps]

    def init(self):
        self.engine.init(self.ladders.ravel())

    def sweep(self, nblocks: int, measure: bool = True):
        """nblocks x (interval Carlo steps of every walker + one exchange step)."""
        acc, prop = self.engine.sweep_tempering(self.ladders, nblocks, self.interval, self.seed, self.step,
                                                measure=measure)
        self.step += nblocks
        self.accepted += acc
        self.proposed += prop

    def temperature_of(self) -> np.ndarray:
        """Current temperature index of every walker, shape (nladders, nrungs)."""
        idx = {t: k for k, t in enumerate(self.temperatures)}
        return np.array([[idx[self.engine.info(int(w))["T"]] for w in row] for row in self.ladders])

    def collect_bin(self):
        """One bin per (ladder, temperature) from the accumulators, which hold the measurements taken at
        the walker's current temperature."""
        where = self.temperature_of()
        for l, row in enumerate(self.ladders):
            out = self.engine.observables(row, reset=True)
            for k, (s, c, _) in enumerate(out):
                self.bins[where[l, k]].append(
                    {n: (s[i] / c[i] if c[i] else np.nan) for i, n in enumerate(self.names)})

    def run(self, sweeps: int, binsize: int):
        """init!, thermalisation (with exchanges), then measured sweeps in bins of `binsize` (rounded up
        to whole exchange intervals)."""
        therm = int(self.params.get("thermalization", 0))
        blocks_per_bin = max(1, -(-int(binsize) // self.interval))
        self.init()
        self.sweep(-(-therm // self.interval) if therm else 0)
        for row in self.ladders:
            self.engine.observables(row, reset=True)
        for _ in range(max(1, sweeps // (blocks_per_bin * self.interval))):
            self.sweep(blocks_per_bin)
            self.collect_bin()

    def acceptance(self) -> np.ndarray:
        """Accepted / proposed swaps per rung pair, summed over ladders."""
        p = self.proposed.sum(0)
        return np.where(p > 0, self.accepted.sum(0) / np.maximum(p, 1), np.nan)

    def results(self) -> list:
        """Per temperature: evaluables with jackknife errors, name -> (mean, error)."""
        return [jackknife_results(b, self.names, self.flat) for b in self.bins]
