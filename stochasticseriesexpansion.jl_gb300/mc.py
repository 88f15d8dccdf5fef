"""Python mirror of the reference's Carlo.jl Monte Carlo interface, backed by the GPU engine.

Reference interface (src/sse.jl):

    MC(params)                       src/sse.jl:26-45
    Carlo.init!(mc, ctx, params)     src/sse.jl:47-60
    Carlo.sweep!(mc, ctx)            src/sse.jl:62-68
    Carlo.measure!(mc, ctx)          src/sse.jl:70-87
    Carlo.write_checkpoint / read_checkpoint   src/sse.jl:89-107
    Carlo.register_evaluables        src/sse.jl:111-134, magnetization_estimator.jl:236-258

``MC`` drives one walker; ``BatchMC`` drives many walkers of one parameter set
in a single persistent launch per sweep block, which is how the engine is
meant to be used.  Both go through ``engine.Engine`` (the C ABI) and raise if
the CUDA library is missing -- there is no CPU fallback.

Parameter names follow the reference: ``T``, ``model`` (a model class such as
``MagnetModel``), ``init_opstring_cutoff``, ``diagonal_warmup_sweeps``,
``init_num_worms``, ``num_worms_attenuation_factor``,
``target_worm_length_fraction``, and the Carlo-level ``thermalization``,
``sweeps``, ``binsize`` and ``seed``.
"""

from __future__ import annotations

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

    @property
    def T(self) -> float:
        return float(self.params["T"])

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
        keys = [k for k in self.names if not all(np.isnan(b[k]) for b in self.bins)]
        arr = {k: np.array([b[k] for b in self.bins]) for k in keys}
        nb = len(self.bins)
        tot = {k: np.nansum(v) for k, v in arr.items()}
        full = evaluables({k: tot[k] / nb for k in keys}, self.flat.est_prefixes, self.flat.norm_site_count)
        loo = [evaluables({k: (tot[k] - arr[k][i]) / (nb - 1) for k in keys}, self.flat.est_prefixes,
                          self.flat.norm_site_count) for i in range(nb)]
        res = {}
        for name, v in full.items():
            x = np.array([l[name] for l in loo])
            res[name] = (v, float(np.sqrt((nb - 1) / nb * np.sum((x - x.mean()) ** 2))))
        for k in keys:
            res.setdefault(k, (float(np.nanmean(arr[k])), float(np.nanstd(arr[k]) / np.sqrt(max(nb, 1)))))
        return res
