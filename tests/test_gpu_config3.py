"""The 2048x512 case (Ra 1e8, contrast 1e6 x 30, 42 M tracers), where the
reference's W-cycle stops with an abnormally high residual
(tests/test_config3_trace.py), solved with the windowed correction
(cycle_correction = 3): the first timesteps run in FP64 and in mixed
precision, every solve meets the 1e-8 test, and the mixed solver's Nu, Vrms
and tracer mass agree with the FP64 solver's within 1e-6 (the error report
over 200 steps is `bench.py --config3 200`)."""
import pytest

from tracer_code_gb300 import Simulation, state

pytestmark = pytest.mark.gpu


def test_config3_converges_with_the_window_in_fp64_and_mixed(gpu_lib):
    import bench
    st = state.initial_state(bench.config3_params(1), seed=1)
    rows = {}
    for prec in (0, 1):
        sim = Simulation(bench.config3_params(prec))
        sim.upload(st)
        rows[prec] = [sim.step() for _ in range(2)]
        sim.close()
    for (ra, qa, _), (rb, qb, _) in zip(rows[1], rows[0]):
        print(f"W-cycles per step: mixed {qa}, FP64 {qb}")
        for k in ("Nu", "vrms"):
            assert ra[k] == pytest.approx(rb[k], rel=1e-6), k
        assert ra["Cavg"][0] == pytest.approx(rb["Cavg"][0], rel=1e-6)
