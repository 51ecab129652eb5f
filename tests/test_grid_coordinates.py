"""The initial state's node coordinates (tracer_code_gb300.state.grid_coordinates,
numpy) are build_grid's (grid.f90:1-109) as the oracle builds them, on the
uniform, arctan and boundary-layer grids: equal on a uniform grid, within the
libm difference (1e-14) on stretched ones."""
import numpy as np
import pytest

from tracer_code_gb300 import state
from tracer_code_gb300.abi import default_params


@pytest.mark.parametrize("gx,gz", [(0, 0), (1, 0), (0, 1), (1, 2), (2, 2)])
def test_initial_state_coordinates_are_build_grids(gx, gz):
    from oracle.pyoracle import Oracle
    p = default_params()
    p.nx, p.nz, p.aspect, p.grids = 64, 32, 2.0, 3
    p.comp, p.tracer = 0, 0
    p.gridX, p.gridZ, p.spaceX, p.spaceZ, p.thickness, p.nbound = gx, gz, 2.0, 1.5, 0.1, 4
    xg, zg = Oracle(p).coordinates()
    x, z = state.grid_coordinates(p)
    # interior nodes (build_grid mirrors its ghosts about the walls)
    xi, zi = xg[3:3 + p.nx + 1], zg[3:3 + p.nz + 1]
    assert np.allclose(x[2:2 + p.nx + 1], xi, rtol=0, atol=1e-14)
    assert np.allclose(z[2:2 + p.nz + 1], zi, rtol=0, atol=1e-14)
    if gx == 0:
        assert np.array_equal(x[2:2 + p.nx], xi[:-1])
    if gz == 0:
        assert np.array_equal(z[2:2 + p.nz], zi[:-1])
    # monotone nodes, ends on the walls
    assert np.all(np.diff(xi) > 0) and np.all(np.diff(zi) > 0)
    assert xi[0] == 0.0 and xi[-1] == p.aspect and zi[0] == 0.0 and zi[-1] == 1.0


@pytest.mark.parametrize("gx,gz", [(0, 0), (1, 0), (0, 1), (1, 2), (2, 1)])
def test_library_metrics_equal_the_oracles(gx, gz):
    """The library's host build of the metrics (tc_grid_metrics: xr, xrr,
    xrrr, xrrrr and DERxr, the same in z) equals the oracle's build_grid bit
    for bit; the kernels read these arrays."""
    import ctypes as C
    from oracle.pyoracle import Oracle
    from tracer_code_gb300 import load_library
    p = default_params()
    p.nx, p.nz, p.aspect, p.grids = 64, 32, 2.0, 3
    p.comp, p.tracer = 0, 0
    p.gridX, p.gridZ, p.spaceX, p.spaceZ, p.thickness, p.nbound = gx, gz, 2.0, 1.5, 0.1, 4
    o = Oracle(p)
    assert (o.nx, o.nz) == (p.nx, p.nz)
    ox, oz = o.metrics()
    L = load_library()
    x5 = np.empty(5 * (p.nx + 7))
    z5 = np.empty(5 * (p.nz + 7))
    assert L.tc_grid_metrics(C.byref(p), x5.ctypes.data_as(C.c_void_p), z5.ctypes.data_as(C.c_void_p)) == 0
    x5, z5 = x5.reshape(5, -1), z5.reshape(5, -1)
    # the reference's ranges: xr, xrr over -1..n+1, the others over 0..n
    for q, lo in zip(range(5), (2, 2, 3, 3, 3)):
        hi = -2 if q < 2 else -3
        assert np.array_equal(x5[q, lo:hi], ox[q, lo:hi]), ("x", q)
        assert np.array_equal(z5[q, lo:hi], oz[q, lo:hi]), ("z", q)


def test_stretched_initial_state_uses_the_physical_coordinates():
    """initialize_tracers / add_tracers on a stretched grid: a tracer is
    enriched where zgrid(s) <= dlayer, a node's C where zg(k) <= dlayer, and
    the temperature profile is evaluated at (xgrid, zgrid) (composition.f90:
    593-664, basics.f90:223-231); on the uniform grid nothing changes."""
    p = default_params()
    p.nx, p.nz, p.aspect, p.tpc, p.dlayer = 32, 16, 2.0, 3, 0.2
    p.gridX, p.gridZ, p.spaceX, p.spaceZ = 1, 1, 2.0, 2.0
    st = state.initial_state(p, seed=4)
    z_tr = state.zgrid(p, st["str"])
    assert np.array_equal(st["Ttype"], np.where(z_tr > p.dlayer, 0, 1))
    x, z = state.grid_coordinates(p)
    assert np.array_equal(st["Cnew"][:, :, 0], np.broadcast_to(np.where(z <= p.dlayer, 1.0, 0.0)[:, None],
                                                                st["Cnew"].shape[:2]))
    T = st["T"]
    span = 2
    k, i = 5, 7
    assert T[span + k, span + i] == (1.0 - z[span + k]) + 0.01 * np.cos(np.pi * x[span + i]) * np.sin(np.pi * z[span + k])
    # the stretching moves the dense layer's boundary off the uniform one
    assert (z_tr <= p.dlayer).sum() != (st["str"] <= p.dlayer).sum()
    u = default_params()
    u.nx, u.nz, u.aspect, u.tpc, u.dlayer = 32, 16, 2.0, 3, 0.2
    su = state.initial_state(u, seed=4)
    assert np.array_equal(su["Ttype"], np.where(su["str"] > u.dlayer, 0, 1))
