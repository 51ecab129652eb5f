"""Cell order of the tracer arrays in HBM (tc_params.tracer_sort_interval; no
reference counterpart).

  - re-sorting the device arrays before every step's RK stages gives the
    same state, statistics and time steps bit for bit as never sorting,
    from a tracer order scrambled at upload;
  - the tracer order seen through the C ABI stays the reference's
    (downloads, tc_step_host);
  - after a re-sort the storage order is the control-volume order that
    tracers_to_corners counts in.
"""
import numpy as np
import pytest

from tracer_code_gb300 import Simulation
from tests.cases import case_1024_like, fresh_state

pytestmark = pytest.mark.gpu


def scrambled(p, seed):
    st = fresh_state(p, seed=seed)
    perm = np.random.default_rng(seed).permutation(len(st["rtr"]))
    for k in ("rtr", "str", "Ttype"):
        st[k] = np.ascontiguousarray(st[k][perm])
    return st


def run(p, st, interval, steps=3):
    q = p.copy()
    q.tracer_sort_interval = interval
    g = Simulation(q)
    g.upload(st)
    rows = [g.step() for _ in range(steps)]
    out = g.download()
    counts = g.counts()
    order = g.tracer_order()
    g.close()
    return rows, out, counts, order


@pytest.mark.parametrize("prec", [0, 1])
def test_sorting_changes_no_result(gpu_lib, prec):
    p = case_1024_like(nx=128, nz=32, grids=4, tpc=4)
    p.solver_precision = prec
    p.mg_zero_coarse = 1
    st = scrambled(p, 5)
    a = run(p, st, 0)
    b = run(p, st, 1)
    assert np.array_equal(a[3], np.arange(len(st["rtr"])))  # never sorted: identity
    assert not np.array_equal(b[3], np.arange(len(st["rtr"])))
    for (ra, qa, dta), (rb, qb, dtb) in zip(a[0], b[0]):
        assert qa == qb and dta == dtb
        for k in ("Nu", "vrms", "Tavg", "Nu_bot"):
            assert ra[k] == rb[k]
        assert ra["Cavg"] == rb["Cavg"]
    for k in ("T", "SF", "Cnew", "rtr", "str", "Ttype"):
        assert np.array_equal(a[1][k], b[1][k]), k
    assert np.array_equal(a[2], b[2])


def test_storage_is_in_cell_order_after_a_sort(gpu_lib):
    p = case_1024_like(nx=128, nz=32, grids=4, tpc=4)
    p.mg_zero_coarse = 1
    p.tracer_sort_interval = 1
    st = scrambled(p, 7)
    g = Simulation(p)
    g.upload(st)
    g.step()
    d = g.download()
    perm = g.tracer_order()
    dr, ds = g.info.dr, g.info.ds
    g.close()
    # the sort ran before step 0's RK stages, on the uploaded positions:
    # their control volumes, in storage order, never decrease
    i = np.floor(st["rtr"][perm] / dr + 0.5).astype(np.int64)
    k = np.floor(st["str"][perm] / ds + 0.5).astype(np.int64)
    cell = k * (p.nx + 1) + i
    assert np.all(np.diff(cell) >= 0)
    assert sorted(perm.tolist()) == list(range(len(perm)))
    assert d["rtr"].shape == st["rtr"].shape


def test_step_host_keeps_reference_order(gpu_lib):
    """tc_step_host (host arrays in, host arrays out) with a re-sort inside
    the step returns the tracers in the order they came in."""
    p = case_1024_like(nx=128, nz=32, grids=4, tpc=4)
    p.mg_zero_coarse = 1
    st = scrambled(p, 9)
    res = []
    for interval in (0, 1):
        q = p.copy()
        q.tracer_sort_interval = interval
        g = Simulation(q)
        g.upload(st)
        hs = {k: np.array(v, copy=True) for k, v in st.items()}
        g.step_host(hs)
        res.append(hs)
        g.close()
    for k in ("rtr", "str", "SF", "T"):
        assert np.array_equal(res[0][k], res[1][k]), k
