"""Restart through a handle (tc_write_restart / tc_read_restart;
print_restart main.f90:301-330 and build_grid's restart branch
grid.f90:55-108).

  - the files a handle writes hold its downloaded state in the reference's
    record layout (xg, zg, T, Cnew, SF; rtr, str, Ttype);
  - a handle restarted from those files is in the same state, and steps to
    the same results bit for bit, as one given the same arrays through
    tc_upload_state.
"""
import struct

import numpy as np
import pytest

from tracer_code_gb300 import Simulation, restart
from tests.cases import case_1024_like, fresh_state

pytestmark = pytest.mark.gpu


def payload(path):
    b = open(path, "rb").read()
    n = struct.unpack("<i", b[:4])[0]
    assert n == len(b) - 8 and struct.unpack("<i", b[-4:])[0] == n
    return b[4:-4]


@pytest.mark.parametrize("prec", [0, 1])
def test_restart_continues_like_upload(gpu_lib, tmp_path, prec):
    p = case_1024_like(nx=128, nz=32, grids=4, tpc=4)
    p.mg_zero_coarse = 1
    p.solver_precision = prec
    a = Simulation(p)
    a.upload(fresh_state(p, seed=11))
    for _ in range(2):
        a.step()
    ta, tt = tmp_path / "Trestart", tmp_path / "restart_tracers"
    a.write_restart(str(ta), str(tt))
    da = a.download()
    nx, nz, ntr = a.nx, a.nz, a.ntr
    a.close()

    # the record layout
    f = np.frombuffer(payload(ta), "<f8")
    xg, zg = restart.grid(nx, nz, p.aspect)
    nf = (nx + 5) * (nz + 5)
    parts = [xg, zg, da["T"].ravel(), da["Cnew"].ravel(), da["SF"].ravel()]
    assert f.size == sum(x.size for x in parts)
    assert np.array_equal(f, np.concatenate(parts))
    assert nf * (2 + p.ntype) + xg.size + zg.size == f.size
    b = payload(tt)
    assert len(b) == 20 * ntr
    assert np.array_equal(np.frombuffer(b[:8 * ntr], "<f8"), da["rtr"])
    assert np.array_equal(np.frombuffer(b[16 * ntr:], "<i4"), da["Ttype"])

    # restart from the files vs upload of the same arrays
    b_ = Simulation(p)
    b_.read_restart(str(ta), str(tt))
    c = Simulation(p)
    c.upload(da)
    db, dc = b_.download(), c.download()
    for k in dc:
        assert np.array_equal(db[k], dc[k]), k
    for _ in range(2):
        rb, qb, tb = b_.step()
        rc, qc, tc = c.step()
        assert qb == qc and tb == tc
        for k in ("Nu", "vrms", "Tavg"):
            assert rb[k] == rc[k]
    db, dc = b_.download(), c.download()
    for k in dc:
        assert np.array_equal(db[k], dc[k]), k
    b_.close()
    c.close()


def test_restart_file_of_another_grid_is_refused(gpu_lib, tmp_path):
    p = case_1024_like(nx=128, nz=32, grids=4, tpc=4)
    a = Simulation(p)
    a.upload(fresh_state(p, seed=2))
    a.write_restart(str(tmp_path / "T"), str(tmp_path / "R"))
    a.close()
    q = case_1024_like(nx=64, nz=32, grids=4, tpc=4)
    b = Simulation(q)
    with pytest.raises(Exception) as e:
        b.read_restart(str(tmp_path / "T"), str(tmp_path / "R"))
    assert getattr(e.value, "status", None) == 1
    with pytest.raises(Exception):
        b.read_restart(str(tmp_path / "T"), None)
    b.close()
