"""Residual trace of the oracle's multigrid on the 2048x512 configuration
(run once on a CPU; the fixture is committed, the oracle is not needed to
read it):

  config_2048x512: aspect 4, 2048x512 cells, 40 tracers per cell
  (42,045,480 tracers), Ra = 1e8, B = 1.0, viscosity contrast 1e6 (T) x 30
  (C), 6 levels, tolerance 1e-8; the seeded initial state (seed 1); the
  first multigrid solve (from SF = 0), capped at CAP W-cycles, once with the
  reference's coarse-level start (mg_zero_coarse = 0) and once with coarse
  corrections restarting from zero (mg_zero_coarse = 1).

Writes tests/golden/config3_trace.json: per setting the level-1 residual
ratio (the quantity the reference's convergence test compares with the
tolerance, iterative_solver.f90:147-156) after every W-cycle, and the status
the capped solve ended with.

    python tests/golden/make_config3_trace.py [CAP]
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import Oracle  # noqa: E402
from tracer_code_gb300 import TracerError, config_2048x512, state  # noqa: E402


def trace(zero: int, cap: int, seed: int = 1, st=None):
    p = config_2048x512()
    p.mg_zero_coarse = zero
    p.max_cycles = cap
    o = Oracle(p)
    o.upload(st if st is not None else state.initial_state(p, seed=seed))
    status = 0
    try:
        o.multigrid()
    except TracerError as e:
        status = e.status
    r = o.residual_trace()
    o.close()
    return [float(v) for v in r], status


def main(cap: int = 60) -> None:
    p = config_2048x512()
    st = state.initial_state(p, seed=1)
    out = {"case": "2048x512", "seed": 1, "cap": cap, "tolerance": p.tolerance, "runs": {}}
    for zero in (0, 1):
        t0 = time.time()
        r, status = trace(zero, cap, st=st)
        out["runs"][str(zero)] = {"mg_zero_coarse": zero, "status": status, "ratios": r}
        print(f"mg_zero_coarse={zero}: {len(r)} cycles, status {status}, last {r[-1]:.3e}, "
              f"min {min(r):.3e} ({time.time() - t0:.0f} s)", flush=True)
    with open(os.path.join(HERE, "config3_trace.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote config3_trace.json")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 60)
