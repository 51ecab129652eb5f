"""Analytic self-checks of the CPU oracle (parts the shipped outputs do not pin)."""
import math

import numpy as np
import pytest

from tracer_code_gb300.abi import Params, default_params, TracerError
from tracer_code_gb300 import state
from oracle.pyoracle import Oracle
from tests.cases import case_128_like, case_1024_like, fresh_state


def test_fd_coefficients_order2():
    p = case_128_like(16, 16, 2, 3)
    o = Oracle(p)
    d = o.fd_coefficients()
    assert d["D1"].tolist()[1:4] == [-0.5, 0.0, 0.5]
    assert d["D2"].tolist()[1:4] == [1.0, -2.0, 1.0]
    assert d["D3"].tolist() == [-0.5, 1.0, 0.0, -1.0, 0.5]
    assert d["D4"].tolist() == [1.0, -4.0, 6.0, -4.0, 1.0]
    assert d["D1_interp"].tolist() == [-0.5, 0.0, 0.5]
    assert d["D2_interp"].tolist() == [1.0, -2.0, 1.0]


def test_derivative_eigenvalue_bounds():
    o = Oracle(case_128_like(16, 16, 2, 3))
    e = o.eig_bases()
    assert e["Tr"] == 1.0 and e["Trr"] == 4.0 and e["Trrrr"] == 16.0
    assert e["Trs"] == 1.0 and e["Trrss"] == 16.0 and e["Trrs"] == 4.0
    # sampled maximum of |sin 2k - 2 sin k| = 3 sqrt(3)/2, single-precision factors
    assert abs(e["Trrr"] - 1.5 * math.sqrt(3)) < 1e-5


def test_cycle_tables_visit_counts():
    o = Oracle(case_1024_like(512, 128, 1, 6))
    info = o.info
    assert info.grids == 6 and info.nsteps == 42
    # W-cycle: level visits 1,3,6,10,14,8 (multigrid_cycle.f90:91-92)


@pytest.mark.parametrize("nx,nz,grids,exp", [(1024, 256, 6, (1024, 256, 6)), (128, 128, 6, (128, 128, 6)),
                                              (2048, 512, 6, (2048, 512, 6)), (200, 200, 2, (200, 200, 2))])
def test_optimize_grid(nx, nz, grids, exp):
    p = case_128_like(nx, nz, 1, grids)
    p.comp = 0
    o = Oracle(p)
    assert (o.nx, o.nz, o.info.grids) == exp


def _manufactured_residual(n):
    p = case_128_like(n, n, 1, 3)
    p.comp = 0
    p.RaT = 1.0
    o = Oracle(p)
    span = 2
    x = np.arange(-span, n + span + 1) / n
    z = np.arange(-span, n + span + 1) / n
    psi = np.sin(np.pi * z)[:, None] * np.sin(np.pi * x)[None, :]
    T = np.ones_like(psi)  # uniform T: zero buoyancy, RHS = 0
    o.upload({"T": T, "SF": psi})
    o.compute_viscosity(1)
    o.compute_rhs(1)
    try:
        o.residual(1, from_sf=True)
    except TracerError as e:  # RHS = 0 makes res_ref = 0, which trips the blow-up guard
        assert e.status == 4
    r = o.get("residual")  # RHS - L psi on the interior
    exact = -(2 * np.pi ** 2) ** 2 * psi[span + 1:span + n, span + 1:span + n]
    return np.max(np.abs(r - exact)) / np.max(np.abs(exact))


def test_operator_converges_second_order():
    e1 = _manufactured_residual(16)
    e2 = _manufactured_residual(32)
    assert e1 < 0.05 and e2 < e1
    assert 3.5 < e1 / e2 < 4.5


def test_multigrid_converges_and_state_is_consistent():
    p = case_128_like(32, 32, 4, 4)
    o = Oracle(p)
    st = fresh_state(p)
    o.upload(st)
    counts = o.counts()
    # sum of counts over the interior box equals the tracer count
    s = 2
    assert counts[s:s + p.nz + 1, s:s + p.nx + 1, :].sum() == o.ntr
    q = o.multigrid()
    assert 1 <= q < 100
    sc = o.scalars()
    assert sc["residual_mag1"] / sc["res_ref1"] <= p.tolerance
    o.compute_velocities()
    row = o.stats()
    assert abs(row["Cavg"][0] - p.dlayer) < 0.05
    assert np.isfinite(row["Nu"]) and row["vrms"] > 0


def test_two_steps_run_and_conserve_tracers():
    p = case_1024_like(128, 32, 3, 4)
    o = Oracle(p)
    o.upload(fresh_state(p))
    for _ in range(2):
        row, q, dt = o.step()
        assert q >= 1 and dt > 0
    out = o.download()
    assert np.all((out["rtr"] > 0) & (out["rtr"] < p.aspect) & (out["str"] > 0) & (out["str"] < 1))
    c = o.counts()
    assert c[2:2 + p.nz + 1, 2:2 + p.nx + 1, :].sum() == o.ntr


def test_zero_coarse_option_converges_on_deep_cycles():
    p = case_1024_like(256, 64, 2, 6, Ra=1e6, visT=1e3)
    p.mg_zero_coarse = 1
    o = Oracle(p)
    o.upload(fresh_state(p))
    q = o.multigrid()
    sc = o.scalars()
    assert sc["residual_mag1"] / sc["res_ref1"] <= p.tolerance and q < 100


def test_tracer_outside_domain_is_reported():
    p = case_128_like(16, 16, 2, 3)
    o = Oracle(p)
    st = fresh_state(p)
    st["rtr"][5] = -0.25
    with pytest.raises(TracerError) as e:
        o.upload(st)
    assert e.value.status == 5


def test_cycle_cap_is_reported():
    p = case_128_like(16, 16, 2, 3)
    p.max_cycles = 1
    p.tolerance = 1e-14
    o = Oracle(p)
    o.upload(fresh_state(p))
    with pytest.raises(TracerError) as e:
        o.multigrid()
    assert e.value.status == 3
