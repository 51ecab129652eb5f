"""Pins the GPU path itself to the reference's shipped outputs (the oracle's
pins in test_oracle_pins.py, run through the C ABI on the device): from
Trestart's T and SF, compute_velocities, compute_strain_rate_invariant,
compute_viscosity(1) (visf with plastic yielding, ivis = 3, and the level-1
viscosity filter) and stats reproduce stats.dat's and
viscosity_smoother.dat's last rows to their 8 printed digits, and as text;
the shipped non-Newtonian solve restarts from Trestart as the oracle does."""
import pytest

from tracer_code_gb300 import Simulation
from tests.test_oracle_pins import _pin_params, _rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu_row(gpu_lib, golden):
    g = Simulation(_pin_params(golden))
    g.upload({"T": golden["T"], "SF": golden["SF"]})
    g.set_clock(0, float(golden["text_lines"]["stats.dat"][-1][:20]))
    g.compute_velocities()
    g.compute_strain()
    g.compute_viscosity(1)
    row = g.stats()
    g.close()
    return row


@pytest.mark.parametrize("col", ["Tavg", "vrms", "Nu", "Nu_bot", "RaT_avg", "mobility", "strain_max",
                                 "q1", "q2", "q3", "q4"])
def test_gpu_stats_row_matches_reference(gpu_row, golden, col):
    ref = golden["stats_last"][col]
    assert _rel(gpu_row[col], ref) < 6e-8, (col, gpu_row[col], ref)


def test_gpu_viscosity_smoother_row_matches_reference(gpu_row, golden):
    ref = golden["viscosity_smoother_last"]
    assert gpu_row["n_eta"] == ref["n_eta"]
    assert gpu_row["n_temp"] == ref["n_temp"]
    assert _rel(gpu_row["eig_fine"], ref["eig_fine"]) < 6e-8


def test_gpu_rows_are_the_reference_text(gpu_row, golden):
    """Written with the reference's formats, the GPU row is the shipped text:
    stats.dat's twelve g20.8 fields (the tracer counts need restart_tracers,
    which is not shipped) and viscosity_smoother.dat's whole row."""
    from tracer_code_gb300 import textio
    RaT = golden["inputs"]["RaT"]
    line = golden["text_lines"]["stats.dat"][-1]
    assert textio.stats_line(gpu_row, 0, 1, 0, RaT)[:240] == line[:240]
    assert textio.vis_line(gpu_row, 0, 0, RaT) == golden["text_lines"]["viscosity_smoother.dat"][-1]


def test_gpu_plastic_solve_from_trestart(gpu_lib, golden):
    """The shipped configuration's non-Newtonian solve (ivis = 3 plastic
    viscosity, non_Newtonian = 1, 2 levels) from Trestart: the stored
    streamfunction is converged, so both sides stop after the first cycle
    and the solution moves by no more than one cycle's smoothing, the same
    on the GPU as in the CPU restatement."""
    import numpy as np
    from oracle.pyoracle import Oracle
    p = _pin_params(golden)
    g = Simulation(p)
    o = Oracle(p)
    for x in (g, o):
        x.upload({"T": golden["T"], "SF": golden["SF"]})
    qg, qo = g.multigrid(), o.multigrid()
    assert qg == qo == 1
    a, b = g.download()["SF"], o.download()["SF"]
    assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max()
    g.close()
