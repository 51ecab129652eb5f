"""The largest configuration at its full size: 2048x512 cells, 40 tracers per
cell (42,045,480 tracers), Ra = 1e8, viscosity contrast 1e6 (T) x 30 (C).
The reference's multigrid does not converge on this case (nor does the CPU
oracle's), so the tracer path is checked on its own, through properties that
do not depend on the size: from a convection-cell streamfunction and one
energy_time with that velocity field held (RK_update = 0), every tracer
stays inside the box, the per-volume counts equal a host recount of the
downloaded positions (nint of r/dr and s/ds, per type), and C is the count
ratio in every volume that holds tracers.
"""
import numpy as np
import pytest

from tracer_code_gb300 import Simulation, config_2048x512, state

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
