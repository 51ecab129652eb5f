"""Temperature tracers (tracer = 1) on the GPU against the CPU oracle, for
comp = 0 (the reference's shipped setting) and comp = 1.

  - upload: Tratio (exact per-volume means of Ttr), counts, T, Cnew bit for
    bit;
  - energy_time with one velocity field for all RK stages (RK_update = 0):
    rtr, str, Ttr, the counts, Tratio and T = Tratio bit for bit (the
    per-volume sums are exact on both sides, so the summation order does
    not matter);
  - full steps (velocities re-solved between stages): stats within 1e-6,
    positions and Ttr within 1e-10;
  - the cell sort carries Ttr with the positions (results unchanged bit for
    bit), and a restart through the reference's files (rtr, str[, Ttype],
    Ttr) continues like an upload.
"""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from tracer_code_gb300 import Simulation, TracerError
from tests.cases import case_1024_like, fresh_state

pytestmark = pytest.mark.gpu

SP = 2


def _case(comp, nx=128, nz=32):
    p = case_1024_like(nx=nx, nz=nz, grids=4, tpc=4)
    p.tracer, p.comp, p.mg_zero_coarse = 1, comp, 1
    return p


def _pair(p, st):
    g, o = Simulation(p), Oracle(p)
    g.upload(st)
    o.upload(st)
    return g, o


@pytest.mark.parametrize("comp", [0, 1])
def test_upload_bitexact(gpu_lib, comp):
    p = _case(comp)
    st = fresh_state(p, seed=4)
    g, o = _pair(p, st)
    assert np.array_equal(g.get("Tratio"), o.get("Tratio"))
    assert np.array_equal(g.counts(), o.counts())
    a, b = g.download(), o.download()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    g.close()


@pytest.mark.parametrize("comp", [0, 1])
def test_energy_time_bitexact_given_identical_velocities(gpu_lib, comp):
    p = _case(comp)
    p.RK_update = 0
    st = fresh_state(p, seed=5)
    g, o = _pair(p, st)
    g.multigrid()
    o.set("SF", g.download()["SF"])
    g.compute_velocities()
    o.compute_velocities()
    assert g.energy_time() == o.energy_time()
    a, b = g.download(), o.download()
    for k in ("rtr", "str", "Ttr", "T") + (("Cnew",) if comp else ()):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(g.counts(), o.counts())
    assert np.array_equal(g.get("Tratio"), o.get("Tratio"))
    ts_g, ts_o = g.get("tracer_space_array"), o.get("tracer_space_array")
    assert np.array_equal(ts_g[1:-1, 1:-1], ts_o)
    g.close()


@pytest.mark.parametrize("comp", [0, 1])
def test_full_steps_parity(gpu_lib, comp):
    p = _case(comp)
    g, o = _pair(p, fresh_state(p, seed=3))
    for n in range(3):
        rg, qg, _ = g.step()
        ro, qo, _ = o.step()
        assert qg == qo
        for key in ("Nu", "vrms", "Tavg", "Nu_bot"):
            assert abs(rg[key] - ro[key]) <= 1e-6 * abs(ro[key]), (n, key, rg[key], ro[key])
        assert (rg["empty_cells"], rg["tracer_min"], rg["tracer_max"]) == \
            (ro["empty_cells"], ro["tracer_min"], ro["tracer_max"])
    a, b = g.download(), o.download()
    for k in ("rtr", "str", "Ttr"):
        assert np.abs(a[k] - b[k]).max() <= 1e-10, k
    g.close()


def test_cell_sort_carries_tracer_temperatures(gpu_lib):
    p = _case(1)
    st = fresh_state(p, seed=7)
    perm = np.random.default_rng(7).permutation(st["rtr"].size)
    for k in ("rtr", "str", "Ttype", "Ttr"):
        st[k] = np.ascontiguousarray(st[k][perm])
    out = []
    for interval in (0, 1):
        q = p.copy()
        q.tracer_sort_interval = interval
        g = Simulation(q)
        g.upload(st)
        rows = [g.step() for _ in range(2)]
        out.append((rows, g.download(), g.tracer_order()))
        g.close()
    assert not np.array_equal(out[1][2], np.arange(st["rtr"].size))
    for (ra, qa, da), (rb, qb, db) in zip(out[0][0], out[1][0]):
        assert qa == qb and da == db and ra["Nu"] == rb["Nu"] and ra["Tavg"] == rb["Tavg"]
    for k in out[0][1]:
        assert np.array_equal(out[0][1][k], out[1][1][k]), k


@pytest.mark.parametrize("comp", [0, 1])
def test_restart_files_with_tracer_temperatures(gpu_lib, tmp_path, comp):
    p = _case(comp)
    a = Simulation(p)
    a.upload(fresh_state(p, seed=2))
    a.step()
    a.write_restart(str(tmp_path / "Trestart"), str(tmp_path / "restart_tracers"))
    da = a.download()
    a.close()
    raw = open(tmp_path / "restart_tracers", "rb").read()
    assert len(raw) == 8 + (28 if comp else 24) * da["rtr"].size
    assert np.array_equal(np.frombuffer(raw[-4 - 8 * da["rtr"].size:-4], "<f8"), da["Ttr"])
    b, c = Simulation(p), Simulation(p)
    b.read_restart(str(tmp_path / "Trestart"), str(tmp_path / "restart_tracers"))
    c.upload(da)
    rb, rc = b.step(), c.step()
    assert rb[1] == rc[1] and rb[2] == rc[2]
    db, dc = b.download(), c.download()
    for k in dc:
        assert np.array_equal(db[k], dc[k]), k
    b.close()
    c.close()


def test_tracer_mode_refuses_host_step_and_plain_upload(gpu_lib):
    p = _case(0)
    st = fresh_state(p, seed=1)
    g = Simulation(p)
    lib = g.L
    import ctypes as C
    T = np.ascontiguousarray(st["T"]); SF = np.ascontiguousarray(st["SF"])
    r = np.ascontiguousarray(st["rtr"]); s = np.ascontiguousarray(st["str"])
    assert lib.tc_upload_state(g.h, T.ctypes.data_as(C.c_void_p), None, SF.ctypes.data_as(C.c_void_p),
                               r.ctypes.data_as(C.c_void_p), s.ctypes.data_as(C.c_void_p), None, r.size) == 1
    g.upload(st)
    with pytest.raises(TracerError) as e:
        g.step_host({k: np.array(v, copy=True) for k, v in st.items()})
    assert e.value.status == 2
    g.close()
