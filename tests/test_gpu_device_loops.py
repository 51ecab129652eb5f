"""The data-dependent loops of a timestep on the device.

The multigrid convergence loop (iterative_solver.f90:105-168) and the three
filter loops -- the viscosity filter smoother_vis (smoother.f90:166-263), the
composition filter smoother_time (:287-341) and the temperature filter
smoother_time_T (:343-377) -- run as CUDA graphs with a WHILE node whose
condition a one-thread test kernel sets after each smoothness / eigenvalue
reduction; the host reads nothing per pass.  With TC_HOST_LOOP set at
creation the same loops run on the host with one read per pass (the
reference's structure).  Both must give the same state bit for bit and the
same filter counts (n_eta, n_temp, n_comp, eig_fine of viscosity_smoother.dat):
  - the 1024x256 physics on a smaller grid (T- and C-dependent viscosity,
    compositional tracers: all three filters), three steps;
  - the reference's shipped configuration on a smaller grid (plastic
    viscosity with the non-Newtonian iteration, temperature tracers), two
    steps.
"""
import os

import numpy as np
import pytest

from tracer_code_gb300 import Simulation
from tests.cases import case_1024_like, fresh_state
from tests.test_gpu_nonnewtonian import _shipped

pytestmark = pytest.mark.gpu

ROW_KEYS = ("Nu", "vrms", "Tavg", "Nu_bot", "n_eta", "n_temp", "eig_fine", "empty_cells", "tracer_min",
            "tracer_max")


def _run(p, st, steps, host_loops):
    if host_loops:
        os.environ["TC_HOST_LOOP"] = "1"
    try:
        g = Simulation(p)
    finally:
        os.environ.pop("TC_HOST_LOOP", None)
    g.upload(st)
    out = [g.step() for _ in range(steps)]
    state = g.download()
    g.close()
    return out, state


@pytest.mark.parametrize("case", ["1024_like", "shipped"])
def test_device_loops_match_host_loops(gpu_lib, case):
    if case == "1024_like":
        p = case_1024_like(nx=128, nz=32, grids=4, tpc=3)
        steps = 3
    else:
        p = _shipped(96, 48, 3)
        steps = 2
    st = fresh_state(p, seed=3)
    dev, sd = _run(p, st, steps, False)
    host, sh = _run(p, st, steps, True)
    for n, ((rd, qd, dtd), (rh, qh, dth)) in enumerate(zip(dev, host)):
        assert qd == qh, (n, qd, qh)
        assert dtd == dth, n
        for k in ROW_KEYS:
            assert rd[k] == rh[k], (n, k, rd[k], rh[k])
        assert list(rd["n_comp"]) == list(rh["n_comp"]), n
        print(f"{case} step {n}: W-cycles {qd}, n_eta {rd['n_eta']}, n_temp {rd['n_temp']}, "
              f"n_comp {list(rd['n_comp'])[:1]}, eig_fine {rd['eig_fine']:.6g}")
    for key in sd:
        assert np.array_equal(sd[key], sh[key]), key
