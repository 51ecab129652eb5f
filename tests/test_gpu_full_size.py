"""The configurations at their full size.

2048x512 cells, 40 tracers per cell (42,045,480 tracers), Ra = 1e8,
viscosity contrast 1e6 (T) x 30 (C): the reference's multigrid does not
converge on this case (nor does the CPU oracle's), so the tracer path is
checked on its own: from a convection-cell streamfunction and one
energy_time with that velocity field held (RK_update = 0), every tracer
stays inside the box, the per-volume counts equal a host recount of the
downloaded positions (nint of r/dr and s/ds, per type), and C is the count
ratio in every volume that holds tracers.

Both full-size configurations (1024x256 with 25 tracers per cell and its
multigrid-solved streamfunction; 2048x512 with the convection cell) against
the CPU oracle from the same state: one energy_time with the velocity field
held gives the same tracer positions, per-volume counts, C and T bit for
bit (the velocities, the Taylor interpolation, the RK updates and the cell
indices are the reference's arithmetic on both sides).
"""
import numpy as np
import pytest

from tracer_code_gb300 import Simulation, config_1024x256, config_2048x512, state

pytestmark = pytest.mark.gpu

SP = 2


def test_full_size_tracer_step_keeps_counts_and_ratio(gpu_lib):
    p = config_2048x512()
    p.RK_update = 0
    st = state.initial_state(p, seed=1)
    x = np.arange(-SP, p.nx + SP + 1) * (p.aspect / p.nx)
    z = np.arange(-SP, p.nz + SP + 1) * (1.0 / p.nz)
    st["SF"] = np.ascontiguousarray(1.0e3 * np.sin(np.pi * z)[:, None] * np.sin(np.pi * x / p.aspect)[None, :])
    g = Simulation(p)
    g.upload(st)
    g.compute_velocities()
    dt = g.energy_time()
    d = g.download()
    counts = g.counts()
    g.close()
    assert dt > 0
    r, s, t = d["rtr"], d["str"], d["Ttype"]
    assert r.size == (p.nx + 1) * (p.nz + 1) * p.tpc
    assert np.all((r > 0) & (r < p.aspect) & (s > 0) & (s < 1))
    assert not np.array_equal(r, st["rtr"])  # the tracers moved
    dr, ds = p.aspect / p.nx, 1.0 / p.nz
    i = np.floor(r / dr + 0.5).astype(np.int64)
    k = np.floor(s / ds + 0.5).astype(np.int64)
    ncell = (p.nx + 1) * (p.nz + 1)
    for ty in range(p.ntype + 1):
        m = t == ty
        host = np.bincount(k[m] * (p.nx + 1) + i[m], minlength=ncell).reshape(p.nz + 1, p.nx + 1)
        assert np.array_equal(host, counts[SP:SP + p.nz + 1, SP:SP + p.nx + 1, ty]), ty
    inner = counts[SP:SP + p.nz + 1, SP:SP + p.nx + 1]
    ne = inner.sum(axis=2)
    ct = inner[:, :, 1]
    C = d["Cnew"][SP:SP + p.nz + 1, SP:SP + p.nx + 1, 0]
    held = ne > 0
    want = np.where(ct == ne, 1.0, np.where(ct == 0, 0.0, ct / np.maximum(ne, 1)))
    assert np.array_equal(C[held], want[held])


def _cell_sf(p):
    x = np.arange(-SP, p.nx + SP + 1) * (p.aspect / p.nx)
    z = np.arange(-SP, p.nz + SP + 1) * (1.0 / p.nz)
    return np.ascontiguousarray(1.0e3 * np.sin(np.pi * z)[:, None] * np.sin(np.pi * x / p.aspect)[None, :])


@pytest.mark.parametrize("size", ["1024x256", "2048x512"])
def test_full_size_energy_time_bitexact_against_oracle(gpu_lib, size):
    from oracle.pyoracle import Oracle
    if size == "1024x256":
        p = config_1024x256()
        p.mg_zero_coarse = 1
    else:
        p = config_2048x512()
    p.RK_update = 0
    st = state.initial_state(p, seed=1)
    if size == "2048x512":
        st["SF"] = _cell_sf(p)
    g = Simulation(p)
    g.upload(st)
    o = Oracle(p)
    o.upload(st)
    if size == "1024x256":
        g.multigrid()
        o.set("SF", g.download()["SF"])
    g.compute_velocities()
    o.compute_velocities()
    dtg = g.energy_time()
    dto = o.energy_time()
    assert dtg == dto
    a, b = g.download(), o.download()
    cg, co = g.counts(), o.counts()
    g.close()
    o.close()
    moved = int(np.count_nonzero(a["rtr"] != st["rtr"]))
    print(f"{size}: {a['rtr'].size} tracers, {moved} moved in r; dt = {dtg:.6e}")
    assert moved > 0
    for key in ("rtr", "str", "Cnew", "T"):
        assert np.array_equal(a[key], b[key]), key
    assert np.array_equal(cg, co)
