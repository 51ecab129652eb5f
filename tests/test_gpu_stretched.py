"""Stretched grids (grid.f90: gridX = 1 arctan; gridZ = 1 arctan, 2 boundary
layers) on the field-temperature path (comp = 0, tracer = 0), the CUDA path
against the oracle on the same seeded inputs:
  - velocities from a given streamfunction: bit for bit (SFx = SFr / xr, SFz =
    SFs / zs at every node);
  - multigrid (arctan stretching; on the boundary-layer grid the oracle's
    W-cycle stops with TC_ERR_MG_RESIDUAL at every setting tried, so gridZ = 2
    is checked through the velocities only): the same W-cycle count,
    |SF_gpu - SF_cpu|_max <= 1e-9 |SF|_max,
    per-level viscosity (its filters use the metric Laplacian) within 1e-12,
    and the GPU solution passes the reference's convergence test under the
    oracle's operator; the mixed solver passes it too;
  - five timesteps: the stats.dat quantities within 1e-6 and the temperature
    within 1e-8;
  - compositional and temperature tracers: velocities divided by the metric
    interpolated at the tracer (interpolate_xr / interpolate_zs), positions,
    counts, C, T and Ttr bit for bit given identical velocities, positions
    within 1e-10 after full steps.
"""
import numpy as np
import pytest

from tracer_code_gb300 import Simulation, TracerError, state
from tracer_code_gb300.abi import default_params
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu

SP = 2


def stretched(gx=1, gz=2, nx=64, nz=32, grids=4, prec=0, Ra=1e5, visT=100.0):
    p = default_params()
    p.nx, p.nz, p.aspect, p.grids = nx, nz, 2.0, grids
    p.comp, p.tracer = 0, 0
    p.gridX, p.gridZ = gx, gz
    p.spaceX, p.spaceZ, p.thickness, p.nbound = 2.0, 1.0, 0.1, 4
    p.RaT = Ra
    p.ivis, p.visT = 2, visT
    p.tolerance = 1e-8
    p.mg_zero_coarse = 1
    p.solver_precision = prec
    return p


def pair(p, st=None):
    g = Simulation(p)
    o = Oracle(p)
    st = state.initial_state(p, seed=1) if st is None else st
    g.upload(st)
    o.upload(st)
    return g, o


def interior(a, nx, nz):
    return a[SP:SP + nz + 1, SP:SP + nx + 1]


@pytest.mark.parametrize("gx,gz", [(1, 0), (0, 1), (1, 2)])
def test_stretched_velocities_bitexact(gpu_lib, gx, gz):
    p = stretched(gx, gz)
    st = state.initial_state(p, seed=1)
    st["SF"] = np.random.default_rng(3).standard_normal(st["T"].shape)
    g, o = pair(p, st)
    g.compute_velocities()
    o.compute_velocities()
    gu, gw = g.velocities()
    ou, ow = o.velocities()
    assert np.array_equal(gu, ou) and np.array_equal(gw, ow)


@pytest.mark.parametrize("gx,gz", [(1, 0), (0, 1), (1, 1)])
def test_stretched_multigrid_parity(gpu_lib, gx, gz):
    p = stretched(gx, gz)
    g, o = pair(p)
    qg = g.multigrid()
    qo = o.multigrid()
    assert qg == qo
    a, b = g.download()["SF"], o.download()["SF"]
    assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max()
    for lev in range(1, g.info.grids + 1):
        nxl, nzl = g.info.nx_grid[lev - 1], g.info.nz_grid[lev - 1]
        va, vb = interior(g.get("vis_grid", lev), nxl, nzl), interior(o.get("vis_grid", lev), nxl, nzl)
        assert np.allclose(va, vb, rtol=1e-12, atol=0), lev
    o.set("SF", a)
    o.compute_rhs(1)
    assert o.residual(1, from_sf=True) / o.reference_residual(1) <= p.tolerance


def test_stretched_mixed_solve_meets_the_tolerance(gpu_lib):
    p = stretched(1, 1, prec=1)
    g, o = pair(p)
    g.multigrid()
    o.multigrid()  # the oracle's operator of this state
    a = g.download()["SF"]
    o.set("SF", a)
    o.compute_rhs(1)
    assert o.residual(1, from_sf=True) / o.reference_residual(1) <= p.tolerance


@pytest.mark.parametrize("gx,gz", [(1, 0), (1, 1)])
def test_stretched_steps_parity(gpu_lib, gx, gz):
    p = stretched(gx, gz)
    g, o = pair(p)
    for n in range(5):
        rg, qg, dtg = g.step()
        ro, qo, dto = o.step()
        assert abs(qg - qo) <= 1, n
        assert dtg == pytest.approx(dto, rel=1e-8)
        for k in ("Nu", "vrms", "Tavg", "Nu_bot", "mobility"):
            assert rg[k] == pytest.approx(ro[k], rel=1e-6), (n, k)
    Tg, To = g.download()["T"], o.download()["T"]
    assert np.abs(Tg - To).max() <= 1e-8


def tracer_case(gx, gz, comp, tracer):
    p = stretched(gx, gz)
    p.comp, p.tracer, p.tpc = comp, tracer, 4
    p.RaC[0] = 0.5 * p.RaT if comp else 0.0
    return p


@pytest.mark.parametrize("gx,gz,comp,tracer", [(1, 0, 1, 0), (1, 1, 0, 1), (0, 1, 0, 1)])
def test_stretched_tracers_bitexact_given_identical_velocities(gpu_lib, gx, gz, comp, tracer):
    """RK_update = 0: one velocity field for all four stages, so both sides
    divide identically interpolated velocities by identically interpolated
    metrics: positions, counts, C and T bit for bit."""
    p = tracer_case(gx, gz, comp, tracer)
    p.RK_update = 0
    g, o = pair(p)
    g.multigrid()
    o.set("SF", g.download()["SF"])
    g.compute_velocities()
    o.compute_velocities()
    assert g.energy_time() == o.energy_time()
    a, b = g.download(), o.download()
    for k in ("rtr", "str", "T"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(g.counts(), o.counts())
    if comp:
        assert np.array_equal(a["Cnew"], b["Cnew"])
    if tracer:
        assert np.array_equal(a["Ttr"], b["Ttr"])


@pytest.mark.parametrize("gx,gz,comp,tracer", [(1, 0, 1, 0), (1, 1, 0, 1)])
def test_stretched_tracer_steps_parity(gpu_lib, gx, gz, comp, tracer):
    p = tracer_case(gx, gz, comp, tracer)
    g, o = pair(p)
    for n in range(3):
        rg, qg, _ = g.step()
        ro, qo, _ = o.step()
        assert abs(qg - qo) <= 1, n
        for k in ("Nu", "vrms", "Tavg"):
            assert rg[k] == pytest.approx(ro[k], rel=1e-6), (n, k)
        if comp:
            assert rg["Cavg"][0] == pytest.approx(ro["Cavg"][0], rel=1e-6)
    a, b = g.download(), o.download()
    assert np.abs(a["rtr"] - b["rtr"]).max() <= 1e-10
    assert np.abs(a["str"] - b["str"]).max() <= 1e-10


def test_stretched_dense_layer_stops_as_the_oracle_does(gpu_lib):
    """comp = 1 with the arctan z-stretching: the oracle's W-cycle stops with
    TC_ERR_MG_RESIDUAL in the first steps; the GPU path stops there too."""
    p = tracer_case(1, 1, 1, 0)
    g, o = pair(p)
    stop = {}
    for side, sim in (("gpu", g), ("oracle", o)):
        try:
            for n in range(3):
                sim.step()
            stop[side] = None
        except TracerError as e:
            stop[side] = (n, e.status)
    assert stop["oracle"] is not None and stop["gpu"] == stop["oracle"]


def test_stretched_coordinates_in_the_handle_and_its_restart_file(gpu_lib, tmp_path):
    """The handle's node coordinates are build_grid's xgrid / zgrid (within
    the libm difference to numpy's), and tc_write_restart writes them."""
    from tracer_code_gb300 import restart
    p = stretched(1, 2)
    g = Simulation(p)
    g.upload(state.initial_state(p, seed=1))
    xg, zg = g.grid_coordinates()
    x, z = state.grid_coordinates(p)
    # interior nodes (the handle's ghosts mirror about the walls)
    assert np.allclose(xg[3:3 + p.nx + 1], x[2:2 + p.nx + 1], rtol=0, atol=1e-14)
    assert np.allclose(zg[3:3 + p.nz + 1], z[2:2 + p.nz + 1], rtol=0, atol=1e-14)
    assert xg[3] == 0.0 and xg[3 + p.nx] == p.aspect and zg[3] == 0.0 and zg[3 + p.nz] == 1.0
    path = str(tmp_path / "Trestart")
    g.write_restart(path)
    d = restart.read_trestart(path, p.nx, p.nz, 0, True)
    assert np.array_equal(d["xg"], xg) and np.array_equal(d["zg"], zg)
    g.close()


@pytest.mark.parametrize("gx,gz", [(1, 0), (0, 1), (1, 2)])
def test_stretched_time_step_tables_bitexact(gpu_lib, gx, gz):
    """The smoothers' pseudo-time steps with the metrics (stability_RK4_smoother,
    stability_vis_smoother) are host tables: bit for bit with the oracle."""
    p = stretched(gx, gz)
    g, o = pair(p)
    # the oracle's arrays cover (0:nx, 0:nz) and (0:a, 0:b), the GPU's the ghost-padded box
    assert np.array_equal(interior(g.get("dts_array"), p.nx, p.nz), o.get("dts_array"))
    for lev in range(1, g.info.grids + 1):
        nxl, nzl = g.info.nx_grid[lev - 1], g.info.nz_grid[lev - 1]
        a = g.get("dt_vis", lev)[SP + 1:SP + nzl, SP:SP + nxl + 1]
        b = o.get("dt_vis", lev)[1:nzl, 0:nxl + 1]
        assert np.array_equal(a, b), lev


@pytest.mark.parametrize("gx,gz", [(1, 0), (1, 1)])
def test_stretched_viscosity_derivatives_and_local_steps(gpu_lib, gx, gz):
    """After a solve's level setup: the metric viscosity derivatives, the
    eigenvalue ratio and the local time step of every level (eigR / eigI with
    the chain rule) against the oracle's, within 1e-10 of each field's largest
    value (the level viscosity agrees to 1e-12, its exp differing in the last
    ulp at most, and differencing amplifies that)."""
    p = stretched(gx, gz)
    g, o = pair(p)
    g.multigrid()
    o.multigrid()
    for lev in range(1, g.info.grids):
        nxl, nzl = g.info.nx_grid[lev - 1], g.info.nz_grid[lev - 1]
        for name in ("vis_x", "vis_z", "vis_xx", "vis_zz", "vis_xz", "dt_stream"):
            a = g.get(name, lev)[SP + 1:SP + nzl, SP + 1:SP + nxl]
            b = o.get(name, lev)  # the oracle's covers the interior (1:a-1, 1:b-1) only
            scale = np.abs(b).max()
            assert np.abs(a - b).max() <= 1e-10 * scale, (lev, name)
