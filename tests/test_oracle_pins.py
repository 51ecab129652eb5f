"""Pins the CPU oracle to the reference's own shipped outputs.

The reference run that produced Trestart ended right after computing
stats.dat's last row and viscosity_smoother.dat's last row from that same
state (main.f90:181-190, then print_restart).  Re-running the oracle's
compute_velocities, compute_strain_rate_invariant, compute_viscosity(1)
(visf ivis=3 + smoother_vis at level 1) and stats on Trestart must therefore
reproduce those rows to the 8 printed digits, and the stored streamfunction
must pass the reference's own convergence test (residual ratio <= the
shipped tolerance) under the oracle's operator.
"""
import numpy as np
import pytest

from tracer_code_gb300.abi import default_params
from oracle.pyoracle import Oracle

pytestmark = []


def _pin_params(g):
    inp = g["inputs"]
    p = default_params()
    p.nx, p.nz, p.aspect, p.order = int(inp["nx"]), int(inp["nz"]), inp["aspect"], int(inp["order"])
    p.comp, p.ntype = int(inp["comp"]), 0
    p.ivis, p.non_Newtonian = int(inp["ivis"]), int(inp["non_Newtonian"])
    p.visT, p.visP, p.delta_visT = inp["visT"], inp["visP"], inp["delta_visT"]
    p.yield_, p.yield_gradient, p.yield_depth = inp["yield"], inp["yield_gradient"], inp["yield_depth"]
    p.RaT, p.tolerance, p.grids, p.Nmulti = inp["RaT"], inp["tolerance"], int(inp["grids"]), int(inp["Nmulti"])
    p.eig_ratio, p.eig_ratio_min, p.vis_iter = inp["eig_ratio"], inp["eig_ratio_min"], int(inp["vis_iter"])
    p.torder, p.courant, p.courantT, p.courant_stream = int(inp["torder"]), inp["courant"], inp["courantT"], inp["courant_stream"]
    p.iterate_order, p.mingrid, p.Tbot, p.Vbc = int(inp["iterate_order"]), int(inp["mingrid"]), int(inp["Tbot"]), int(inp["Vbc"])
    return p


@pytest.fixture(scope="module")
def pinned(golden):
    p = _pin_params(golden)
    o = Oracle(p)
    o.upload({"T": golden["T"], "SF": golden["SF"]})
    o.compute_velocities()
    o.compute_strain()
    o.compute_viscosity(1)
    return o


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def test_grid_coordinates_match_restart(pinned, golden):
    # the restart file's zg equals the uniform grid the oracle builds
    ds = 1.0 / 200
    z = golden["zg"][3:3 + 201]
    assert np.array_equal(z, ds * np.arange(201))


@pytest.mark.parametrize("col", ["Tavg", "vrms", "Nu", "Nu_bot", "RaT_avg", "mobility", "strain_max",
                                 "q1", "q2", "q3", "q4"])
def test_stats_row_matches_reference(pinned, golden, col):
    row = pinned.stats()
    ref = golden["stats_last"][col]
    # stats.dat prints g20.8: 8 significant digits
    assert _rel(row[col], ref) < 6e-8, (col, row[col], ref)


def test_viscosity_smoother_row_matches_reference(pinned, golden):
    sc = pinned.scalars()
    ref = golden["viscosity_smoother_last"]
    assert int(sc["n_eta"]) == ref["n_eta"]
    assert int(sc["n_temp"]) == ref["n_temp"]
    assert _rel(sc["eig_fine"], ref["eig_fine"]) < 6e-8


def test_restart_streamfunction_passes_reference_convergence_test(pinned, golden):
    o = pinned
    o.compute_rhs(1)
    ref = o.reference_residual(1)
    res = o.residual(1, from_sf=True)
    tol = golden["inputs"]["tolerance"]
    assert res / ref <= tol
    # the check has teeth: a 1% perturbation of SF fails it by far
    SF = golden["SF"].copy() * 1.01
    o.set("SF", SF)
    bad = o.residual(1, from_sf=True)
    assert bad / ref > 5 * tol
    o.set("SF", golden["SF"])


def test_stats_and_viscosity_lines_match_reference_text(pinned, golden):
    """The recomputed row, written with the reference's formats
    (tc_format_stats_line / tc_format_vis_line), is the shipped text: the
    twelve g20.8 fields of stats.dat's last row (its three tracer counts need
    restart_tracers, which is not shipped) and the whole last row of
    viscosity_smoother.dat."""
    from tracer_code_gb300 import build as tcbuild
    tcbuild.build()
    from tracer_code_gb300 import textio
    line = golden["text_lines"]["stats.dat"][-1]
    row = pinned.stats()
    row["time"] = float(line[:20])
    assert textio.stats_line(row, 0, 1, 0, golden["inputs"]["RaT"])[:240] == line[:240]
    sc = pinned.scalars()
    vl = golden["text_lines"]["viscosity_smoother.dat"][-1]
    r2 = {"time": float(vl[:20]), "n_eta": int(sc["n_eta"]), "eig_fine": sc["eig_fine"], "n_temp": int(sc["n_temp"])}
    assert textio.vis_line(r2, 0, 0, golden["inputs"]["RaT"]) == vl
