"""T1xxxx snapshot of a handle (tc_write_snapshot; snapshots, main.f90:237-270).

Every line of the file is the reference's '(9(g14.5E3),i6,20(g14.5E3))'
record of one node, in the reference's order (i outer, k inner, a blank
list-directed record after each i), holding the handle's state as the
downloads and diagnostic copies give it: xg, zg, T, SF, u, w, strain, vis
(level-1 vis_grid, which stats copies into vis), Tvis, nempty, Cnew, Cvis.
"""
import numpy as np
import pytest

from tracer_code_gb300 import Simulation, restart, textio
from tests.cases import case_1024_like, fresh_state

pytestmark = pytest.mark.gpu


def test_snapshot_lines_hold_the_state(gpu_lib, tmp_path):
    p = case_1024_like(nx=128, nz=32, grids=4, tpc=4)
    p.mg_zero_coarse = 1
    g = Simulation(p)
    g.upload(fresh_state(p, seed=5))
    g.step()
    g.multigrid()
    g.compute_velocities()
    g.stats()
    path = tmp_path / "T10001"
    g.write_snapshot(str(path))
    nx, nz, nt = g.nx, g.nz, p.ntype
    d = g.download()
    u, w = g.velocities()
    strain, vis, Tvis = g.get("strain", 1), g.get("vis_grid", 1), g.get("Tvis", 1)
    Cvis = [g.get("Cvis", 1, t + 1) for t in range(nt)]
    nempty = g.counts().sum(axis=2)
    g.close()
    xg, zg = restart.grid(nx, nz, p.aspect)

    lines = open(path).read().split("\n")
    assert lines[-1] == ""
    lines = lines[:-1]
    assert len(lines) == (nx + 1) * (nz + 2)
    f = lambda v: textio.format_g(v, 14, 5, 3)
    n = 0
    for i in range(nx + 1):
        for k in range(nz + 1):
            line = lines[n]
            n += 1
            want = "".join(f(v) for v in (xg[i + 3], zg[k + 3], d["T"][k + 2, i + 2], d["SF"][k + 2, i + 2],
                                           u[k + 1, i + 1], w[k + 1, i + 1], strain[k + 2, i + 2],
                                           vis[k + 2, i + 2], Tvis[k + 2, i + 2]))
            want += f"{int(nempty[k + 2, i + 2]):6d}"
            want += "".join(f(d["Cnew"][k + 2, i + 2, t]) for t in range(nt))
            want += "".join(f(Cvis[t][k + 2, i + 2]) for t in range(nt))
            assert line == want, (i, k)
        assert lines[n] == "  "
        n += 1
    # the values are the state's, not placeholders
    assert np.abs(u).max() > 0 and nempty[2:-2, 2:-2].min() >= 0 and nempty.max() > 0
