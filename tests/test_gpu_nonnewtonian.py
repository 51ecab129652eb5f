"""The reference's shipped configuration on the GPU: plastic viscosity
(ivis = 3) with the non-Newtonian multigrid iteration (non_Newtonian = 1:
velocities, strain rate, every level's viscosity, local time steps and the
coarse LU rebuilt each W-cycle, the level-1 viscosity and residual brought
up to date before the convergence test; iterative_solver.f90:79-173) and
temperature tracers (tracer = 1, comp = 0), on smaller grids, against the
CPU oracle:
  - one solve: same cycle count, streamfunction within 1e-9 of its maximum;
  - full steps: same cycle counts, stats within 1e-6, tracer positions and
    temperatures within 1e-10.
"""
import json
import os

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from tracer_code_gb300 import Simulation
from tests.cases import fresh_state
from tests.test_oracle_pins import _pin_params

pytestmark = pytest.mark.gpu


def _shipped(nx, nz, grids):
    with open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")) as f:
        p = _pin_params(json.load(f))
    p.tracer, p.nx, p.nz, p.grids, p.tpc = 1, nx, nz, grids, 4
    return p


@pytest.mark.parametrize("nx,nz,grids", [(64, 64, 2), (96, 48, 3), (128, 64, 4)])
def test_nonnewtonian_solve_parity(gpu_lib, nx, nz, grids):
    p = _shipped(nx, nz, grids)
    st = fresh_state(p, seed=1)
    g, o = Simulation(p), Oracle(p)
    g.upload(st)
    o.upload(st)
    assert g.multigrid() == o.multigrid()
    a, b = g.download()["SF"], o.download()["SF"]
    assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max()
    g.close()


@pytest.mark.parametrize("nx,nz,grids", [(64, 64, 2), (96, 48, 3)])
def test_nonnewtonian_steps_parity(gpu_lib, nx, nz, grids):
    p = _shipped(nx, nz, grids)
    st = fresh_state(p, seed=2)
    g, o = Simulation(p), Oracle(p)
    g.upload(st)
    o.upload(st)
    for n in range(2):
        rg, qg, _ = g.step()
        ro, qo, _ = o.step()
        assert qg == qo, n
        for key in ("Nu", "vrms", "Tavg", "Nu_bot", "strain_max"):
            assert abs(rg[key] - ro[key]) <= 1e-6 * abs(ro[key]), (n, key, rg[key], ro[key])
        assert rg["n_eta"] == ro["n_eta"] and rg["n_temp"] == ro["n_temp"]
    a, b = g.download(), o.download()
    for k in ("rtr", "str", "Ttr"):
        assert np.abs(a[k] - b[k]).max() <= 1e-10, k
    g.close()


def test_nonnewtonian_refuses_mixed_precision(gpu_lib):
    from tracer_code_gb300 import TracerError
    p = _shipped(64, 64, 2)
    p.solver_precision = 1
    with pytest.raises(TracerError) as e:
        Simulation(p)
    assert e.value.status == 2
