"""bench.py's default run end to end on the CPU: the engine is the emulated-warp build of
tests/warp_emu (the real kernels' logic, on emulated warps) and the sizes are tiny.  The numbers
are meaningless here (the emulated runtime's clock is not the GPU's); what is checked is that the
run completes and prints one JSON line with every key the benchmark contract asks for, in the
right types.  The measured line itself comes from a GB300."""

import json

import pytest

REQUIRED = {
    "metric": str, "value": float, "unit": str, "n_gpus": int, "steps": int, "warmup": int, "ms_per_step": float,
    "higher_is_better": bool, "scaling": str, "dtype": str, "data": str, "config": dict, "roofline": dict,
    "cpu_baseline": dict, "e2e": dict, "gpu_launches": int, "clocks": dict,
}


def test_bench_default_run_prints_the_contract_line(S, emu, monkeypatch, capsys):
    import importlib.util
    import os

    import sse_gb300.engine as E

    real_init = E.Engine.__init__

    def emulated(self, device=0, library=None):
        real_init(self, device, library if library is not None else emu)

    monkeypatch.setattr(E.Engine, "__init__", emulated)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("_bench_under_test", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    monkeypatch.setattr("sys.argv", ["bench.py", "--walkers", "6", "--side", "4", "--beta", "2", "--therm", "4",
                                     "--steps", "2", "--warmup", "3", "--sweeps-per-step", "2",
                                     "--plain-walkers", "2", "--cpu-sweeps", "4", "--cpu-threads", "2",
                                     "--serving-requests", "0"])
    bench.main()
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key, typ in REQUIRED.items():
        assert key in line, key
        assert isinstance(line[key], typ) or (typ is float and isinstance(line[key], int)), (key, line[key])
    assert line["vs_baseline"] is None and line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["value"] > 0 and line["gpu_launches"] >= line["steps"]
    for key in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert key in line["roofline"], key
    for key in ("value", "unit", "cores", "kind", "sample"):
        assert key in line["cpu_baseline"], key
    assert line["cpu_baseline"]["kind"] == "port"
    for key in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert key in line["e2e"], key
    assert line["e2e"]["h2d_bytes_per_step"] > 0 and line["e2e"]["d2h_bytes_per_step"] > 0
    assert "workload" in line["config"]
    for key in ("sm_mhz", "sm_max_mhz", "reasons"):
        assert key in line["clocks"], key


def test_smoke_runs_against_the_oracle(S, emu, monkeypatch):
    """__graft_entry__.smoke() (4 walkers of the 8x8 model, init plus 6 Carlo steps, checked
    against the oracle) completes on the emulated engine: its checks hold for the kernels' logic."""
    import importlib.util
    import os

    import sse_gb300.engine as E

    real_init = E.Engine.__init__
    monkeypatch.setattr(E.Engine, "__init__",
                        lambda self, device=0, library=None: real_init(self, device, library if library else emu))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("_entry_under_test", os.path.join(root, "__graft_entry__.py"))
    entry = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(entry)
    entry.smoke()


def test_reference_task_workload_prints_its_line(S, emu, monkeypatch, capsys):
    """--workload magnet_bench (the reference's own benchmark task, batched) on two tiny walkers:
    one JSON line with the batched, single-walker and CPU rates and the worm-cap accounting."""
    import importlib.util
    import os

    import sse_gb300.engine as E

    real_init = E.Engine.__init__
    monkeypatch.setattr(E.Engine, "__init__",
                        lambda self, device=0, library=None: real_init(self, device, library if library else emu))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("_bench_under_test2", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    monkeypatch.setattr("sys.argv", ["bench.py", "--workload", "magnet_bench", "--walkers", "2", "--therm", "5",
                                     "--steps", "1", "--sweeps-per-step", "3", "--cpu-sweeps", "2",
                                     "--cpu-threads", "2"])
    bench.main()
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key in ("workload", "walkers", "walkers_stopped_by_worm_cap", "thermalisation_sweeps_undone_at_worm_cap",
                "gpu_batched_walker_sweeps_per_s", "gpu_single_walker_sweeps_per_s",
                "cpu_oracle_all_cores_walker_sweeps_per_s"):
        assert key in line, key
    assert line["workload"] == "magnet_bench" and line["walkers"] == 2
