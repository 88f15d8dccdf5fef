"""Writes the golden trajectory fixtures:

* tests/golden/model_<case>.npz   the flattened model tables of each case.  The LP behind S >= 1
  tables may pick another optimal vertex, or differ in the last bits, on another machine or
  solver version, so the fixtures carry the tables themselves.
* tests/golden/trajectories.json  for seeded walkers of each case, run by the CPU oracle from
  Carlo.init! for a number of Carlo steps: opstring and spin-state digests (sha256 of the
  little-endian uint32 / uint8 arrays), the scalar chain state and the observable sums (exact hex
  floats).

The tests check that the oracle still reproduces these values from the stored tables and that the
GPU engine reaches them.

    python tests/golden/make_golden.py
"""

import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

import _sse_loader  # noqa: E402

S = _sse_loader.load()
from oracle import oracle as O  # noqa: E402
from golden_cases import CASES, save_flat  # noqa: E402


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_case(name, case):
    flat = S.flatten_model(case["model"](S))
    save_flat(flat, os.path.join(HERE, f"model_{name}.npz"))
    om = O.OracleModel(flat)
    out = []
    for stream in case["streams"]:
        w = O.OracleWalker(om, T=case["T"], seed=case["seed"], stream=stream, thermalization=case["therm"])
        w.init()
        w.run(case["sweeps"], measure=True)
        s, c, _ = w.obs()
        out.append({
            "stream": stream,
            "L": int(w.w.L), "n": int(w.w.num_operators), "rng_counter": int(w.w.ctr),
            "num_worms": float(w.w.num_worms).hex(), "avg_worm_length": float(w.w.avg_worm_length).hex(),
            "ops_sha256": digest(w.ops.astype("<u4")), "state_sha256": digest(w.state.astype(np.uint8)),
            "obs_sums": [float(x).hex() for x in s], "obs_counts": [int(x) for x in c],
        })
    return out


if __name__ == "__main__":
    data = {name: {"T": c["T"], "seed": c["seed"], "therm": c["therm"], "sweeps": c["sweeps"],
                   "walkers": run_case(name, c)} for name, c in CASES.items()}
    with open(os.path.join(HERE, "trajectories.json"), "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", len(data), "cases")
