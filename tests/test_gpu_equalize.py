"""Tracer repositioning, TRA (equalize = 1; equalize_tracers,
composition.f90:83-580) on the GPU against the oracle, reproducing the
reference run with 1, 4 and 7 OpenMP threads (mzran streams and static
loop shares per thread):

  - one energy_time from an uneven tracer distribution with identical
    velocities (RK_update = 0): the equalize.dat values, every tracer's
    position, type and temperature, the counts, C and T bit for bit;
  - full steps: the equalize.dat rows equal, stats within 1e-6.
"""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from tracer_code_gb300 import Simulation
from tracer_code_gb300.state import initial_tracer_temperature, uniforms
from tests.cases import case_1024_like, fresh_state

pytestmark = pytest.mark.gpu


def _case(comp, tracer, NR, nx=64, nz=32):
    p = case_1024_like(nx=nx, nz=nz, grids=3, tpc=4)
    p.comp, p.tracer, p.mg_zero_coarse = comp, tracer, 1
    p.equalize, p.equalize_threads = 1, NR
    return p


def _uneven(p, seed):
    """fresh_state with the tracers spread uniformly over the box instead
    of tpc per volume, so that volumes hold uneven counts"""
    st = fresh_state(p, seed=seed)
    n = st["rtr"].size
    ids = np.arange(n, dtype=np.int64)
    st["rtr"] = np.ascontiguousarray(0.001 + (p.aspect - 0.002) * uniforms(seed + 7, ids, 0))
    st["str"] = np.ascontiguousarray(0.001 + 0.998 * uniforms(seed + 7, ids, 1))
    if p.comp == 1:
        st["Ttype"] = np.ascontiguousarray(np.where(st["str"] > p.dlayer, 0, 1).astype(np.int32))
    if p.tracer == 1:
        st["Ttr"] = initial_tracer_temperature(st["rtr"], st["str"])
    return st


@pytest.mark.parametrize("comp,tracer", [(0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("NR", [1, 4, 7])
def test_equalize_bitexact_given_identical_velocities(gpu_lib, comp, tracer, NR):
    p = _case(comp, tracer, NR)
    p.RK_update = 0
    st = _uneven(p, 3)
    g, o = Simulation(p), Oracle(p)
    g.upload(st)
    o.upload(st)
    g.multigrid()
    o.set("SF", g.download()["SF"])
    for x in (g, o):
        x.set_clock(0, 0.0)
        x.compute_velocities()
        x.stats()  # Cinit at time 0
    assert g.energy_time() == o.energy_time()
    rg, ro = g.equalize_row(), o.equalize_row()
    assert rg == ro and len(rg) > 0 and rg[-1 - (p.ntype if comp else 0) - 2] > 0, (rg, ro)
    a, b = g.download(), o.download()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(g.counts(), o.counts())
    g.close()


@pytest.mark.parametrize("comp,tracer", [(0, 1), (1, 0)])
def test_equalize_full_steps(gpu_lib, comp, tracer):
    p = _case(comp, tracer, 4, nx=128, nz=32)
    st = _uneven(p, 5)
    g, o = Simulation(p), Oracle(p)
    g.upload(st)
    o.upload(st)
    for n in range(3):
        rg, qg, _ = g.step()
        ro, qo, _ = o.step()
        assert qg == qo
        assert g.equalize_row() == o.equalize_row(), n
        for key in ("Nu", "vrms", "Tavg"):
            assert abs(rg[key] - ro[key]) <= 1e-6 * abs(ro[key]), (n, key)
        assert (rg["empty_cells"], rg["tracer_min"], rg["tracer_max"]) == \
            (ro["empty_cells"], ro["tracer_min"], ro["tracer_max"])
    g.close()
