"""Mixed-precision multigrid (solver_precision=1): FP32 smoother and coarse
levels inside an FP64 defect-correction loop.

There is no reference counterpart; its judge is the reference's own
convergence test, evaluated by the CPU oracle in FP64 on the GPU result:
  - relative L1 residual (iterative_solver.f90:155) <= tolerance;
  - streamfunction within 1e-6 |SF|_max of the FP64 oracle solution (both
    satisfy the same residual tolerance, so they differ by the solve error,
    not by rounding);
  - W-cycle count within 20% (+1) of the FP64 solve;
  - over several full steps Nu, Vrms and mass within 1e-6 relative of the
    FP64 oracle, and the per-cell tracer counts identical.
"""
import numpy as np
import pytest

from tracer_code_gb300 import Simulation
from tracer_code_gb300.abi import config_1024x256
from tests.cases import case_128_like, case_1024_like, fresh_state
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def _mixed(p):
    q = p.copy()
    q.solver_precision = 1
    return q


def _residual_ratio(o, sf):
    o.set("SF", sf)
    o.compute_rhs(1)
    ref = o.reference_residual(1)
    return o.residual(1, from_sf=True) / ref


@pytest.mark.parametrize("mk,zero", [(case_128_like, 0), (case_1024_like, 0), (case_1024_like, 1)])
def test_mixed_multigrid_meets_reference_tolerance(gpu_lib, mk, zero):
    p = mk()
    p.mg_zero_coarse = zero
    st = fresh_state(p)
    g = Simulation(_mixed(p))
    g.upload(st)
    o = Oracle(p)
    o.upload(st)
    qg = g.multigrid()
    qo = o.multigrid()
    a, b = g.download()["SF"], o.download()["SF"]
    assert abs(qg - qo) <= 0.2 * qo + 1, (qg, qo)
    assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()
    assert _residual_ratio(o, a) <= p.tolerance


def test_mixed_multigrid_full_contrast(gpu_lib):
    """The 1024x256 case's physics at full contrast (visT=1e4, Ra=1e7) on a
    512x128 grid with 6 levels: the FP64 oracle's residual test passes on
    the mixed solution, and the FP64 GPU solve takes a similar cycle count."""
    p = config_1024x256()
    p.nx, p.nz, p.tpc, p.grids = 512, 128, 2, 6
    p.mg_zero_coarse = 1
    st = fresh_state(p)
    g64 = Simulation(p)
    g64.upload(st)
    q64 = g64.multigrid()
    g32 = Simulation(_mixed(p))
    g32.upload(st)
    q32 = g32.multigrid()
    assert abs(q32 - q64) <= 0.2 * q64 + 1, (q32, q64)
    o = Oracle(p)
    o.upload(st)
    o.compute_viscosity(1)
    assert _residual_ratio(o, g32.download()["SF"]) <= p.tolerance


def test_mixed_steps_against_fp64_oracle(gpu_lib):
    p = case_1024_like()
    st = fresh_state(p)
    g = Simulation(_mixed(p))
    g.upload(st)
    o = Oracle(p)
    o.upload(st)
    for n in range(3):
        rg, _, _ = g.step()
        ro, _, _ = o.step()
        for key in ["Nu", "vrms"]:
            assert abs(rg[key] - ro[key]) <= 1e-6 * abs(ro[key]), (n, key, rg[key], ro[key])
        assert abs(rg["Cavg"][0] - ro["Cavg"][0]) <= 1e-6 * abs(ro["Cavg"][0])
    assert np.array_equal(g.counts(), o.counts())
    a, b = g.download(), o.download()
    assert np.abs(a["rtr"] - b["rtr"]).max() <= 1e-8
    assert np.abs(a["str"] - b["str"]).max() <= 1e-8


def _capped_correction(p, st, fields=None):
    # two W-cycles at most: the level-1 correction after the first cycle's
    # coarse work and the second cycle's level-1 visit
    from tracer_code_gb300 import TracerError
    q = p.copy()
    q.tolerance, q.max_cycles = 1e-300, 2
    g = Simulation(q)
    g.upload(st)
    if fields is not None:
        g.debug_sweep_fields(fields)
    with pytest.raises(TracerError):
        g.multigrid()
    e1 = g.get("error", 1)
    g.close()
    return e1


def test_level1_field_sweep(gpu_lib):
    """The level-1 FP32 sweep that forms its coefficients from five FP32
    viscosity fields is as close to the FP64 cycle as the sweep over the
    13 coefficient planes rounded from FP64, and the full solves meet the
    oracle's residual test with W-cycle counts within 10% (+1) of each
    other."""
    p = case_1024_like(nx=256, nz=64, grids=5, tpc=3)
    p.mg_zero_coarse = 1
    st = fresh_state(p, seed=7)
    a = _capped_correction(p, st)
    m = _mixed(p)
    ef = _capped_correction(m, st, fields=True)
    ep = _capped_correction(m, st, fields=False)
    scale = np.abs(a).max()
    df, dp = np.abs(ef - a).max() / scale, np.abs(ep - a).max() / scale
    print(f"one cycle against FP64: field sweep {df:.3e}, coefficient planes {dp:.3e}")
    assert df <= 2.0 * dp + 1e-12
    cyc, sf = {}, {}
    for fields in (True, False):
        g = Simulation(m)
        g.upload(st)
        g.debug_sweep_fields(fields)
        cyc[fields] = g.multigrid()
        sf[fields] = g.download()["SF"]
        g.close()
    print(f"W-cycles: field sweep {cyc[True]}, coefficient planes {cyc[False]}")
    assert abs(cyc[True] - cyc[False]) <= 0.1 * cyc[False] + 1
    o = Oracle(p)
    o.upload(st)
    o.compute_viscosity(1)
    assert _residual_ratio(o, sf[True]) <= p.tolerance
    o.close()


def test_field_sweep_toggle_needs_mixed(gpu_lib):
    from tracer_code_gb300 import TracerError
    p = case_128_like()
    g = Simulation(p)
    g.upload(fresh_state(p, seed=1))
    with pytest.raises(TracerError):
        g.debug_sweep_fields(False)
    g.close()


@pytest.mark.parametrize("nx,nz", [(256, 64), (200, 72)])
def test_level1_tiled_field_sweeps_bit_exact(gpu_lib, nx, nz):
    """Two or three level-1 field sweeps per launch (k_sweep_gblk, 64x16
    tiles with recomputed halos, coefficients in shared memory) give the
    one-sweep-per-launch result bit for bit, on grids whose interior is not
    a multiple of the tile (partial tiles at the far walls)."""
    p = _mixed(case_1024_like(nx=nx, nz=nz, grids=4, tpc=3))
    p.mg_zero_coarse = 1
    st = fresh_state(p, seed=11)
    g0 = Simulation(p)
    g0.upload(st)
    base = g0.autotune()
    g0.close()
    sf = {}
    for blk in (0, 2, 3):
        shapes = [list(c) for c in base]
        shapes[0][2] = 1000 + blk if blk else 0
        g = Simulation(p)
        g.upload(st)
        g.set_launch_shapes(shapes)
        q = g.multigrid()
        sf[blk] = (q, g.download()["SF"])
        g.close()
    for blk in (2, 3):
        assert sf[blk][0] == sf[0][0], (blk, sf[blk][0], sf[0][0])
        assert np.array_equal(sf[blk][1], sf[0][1]), blk
