"""The 2048x512 configuration (Ra = 1e8, contrast 1e6 x 30, 6 levels) does
not converge under the reference's multigrid, on the CPU oracle itself (the
windowed correction makes it converge: tests/test_gpu_config3.py).

tests/golden/make_config3_trace.py ran the oracle's first solve of the
seeded state (capped W-cycles, both coarse-level starts) and committed the
level-1 residual ratio after every cycle.  This test holds that record to
what it shows and re-derives its first cycles:

  - neither run reaches the 1e-8 tolerance within its cap; over the last
    half of each run the ratio never falls below 1e-4 (it stalls or grows,
    no geometric decay);
  - the oracle, run again here for two W-cycles on the full-size state,
    reproduces the first two recorded ratios (to 1e-12 relative).
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(__file__), "golden")
FIXTURE = os.path.join(HERE, "config3_trace.json")


def _load():
    with open(FIXTURE) as f:
        return json.load(f)


@pytest.mark.skipif(not os.path.exists(FIXTURE), reason="fixture not generated")
def test_recorded_trace_does_not_converge():
    d = _load()
    for key, run in d["runs"].items():
        r = np.array(run["ratios"])
        assert r.size >= 2, key
        assert r.min() > 100 * d["tolerance"], (key, r.min())
        tail = r[r.size // 2:]
        assert tail.min() > 1e-4, (key, tail.min())
        assert run["status"] != 0, key  # the capped solve stopped (cycle cap or diverging residual)
        print(f"mg_zero_coarse={run['mg_zero_coarse']}: {r.size} cycles, first {r[0]:.3e}, "
              f"min {r.min():.3e}, last {r[-1]:.3e}, status {run['status']}")


@pytest.mark.skipif(not os.path.exists(FIXTURE), reason="fixture not generated")
def test_first_cycles_rederived():
    from tests.golden.make_config3_trace import trace
    d = _load()
    for key, run in d["runs"].items():
        r, _ = trace(int(run["mg_zero_coarse"]), cap=2, seed=d["seed"])
        assert len(r) == 2
        want = np.array(run["ratios"][:2])
        assert np.allclose(r, want, rtol=1e-12, atol=0.0), (key, r, want)
