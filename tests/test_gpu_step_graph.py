"""The timestep as one CUDA graph launch (tc_set_step_graph, tc_ensemble_run).

A captured step replays the eager step's kernels with the multigrid
convergence loop and the filter loops as conditional WHILE nodes, and does
the eager step's reads of the device scalars after the launch.  So:
  - every step's stats row, W-cycle count and dt, and the state after the
    run, equal the eager handle's bit for bit (FP64 and mixed solver,
    windowed correction, across a tracer sort, with the learned start and
    direction);
  - a step that fails returns the eager step's status and cycle count;
  - an ensemble stepped by one graph launch per step ends where its cases
    end when stepped alone, and its later steps are graph launches.
"""
import os

import numpy as np
import pytest

from tracer_code_gb300 import Simulation, TracerError, state
from tracer_code_gb300.abi import config_1024x256

pytestmark = pytest.mark.gpu

WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tracer_code_gb300", "weights",
                       "guess_512x128.npy")


def case(nx=256, nz=64, grids=4, prec=1, Ra=1e6, visT=1e3, tpc=4, cc=3):
    p = config_1024x256()
    p.nx, p.nz, p.grids, p.tpc = nx, nz, grids, tpc
    p.RaT = Ra
    p.RaC[0] = 0.6 * Ra
    p.visT = visT
    p.mg_zero_coarse = 1
    p.mg_coarse_matrix = 1
    p.solver_precision = prec
    p.cycle_correction = cc
    return p


def run(p, seed, steps, graph, weights=None):
    from tracer_code_gb300 import learned
    sim = Simulation(p)
    net = None
    if weights:
        net = learned.Net(1, p.nz, p.nx)
        net.load(weights)
        learned.attach(sim, net)
    sim.upload(state.initial_state(p, seed=seed))
    if graph:
        sim.set_step_graph(True)
    out = [sim.step() for _ in range(steps)]
    d = sim.download()
    info = sim.step_graph_info()
    sim.close()
    if net:
        net.close()
    return out, d, info


def assert_same(a, b):
    (ra, da, _), (rb, db, _) = a, b
    for (row_a, qa, dta), (row_b, qb, dtb) in zip(ra, rb):
        assert qa == qb and dta == dtb
        assert row_a == row_b
    for k in ("T", "SF", "rtr", "str", "Ttype"):
        assert np.array_equal(da[k], db[k]), k


@pytest.mark.parametrize("prec,cc", [(1, 3), (0, 0), (1, 0)])
def test_graph_steps_equal_eager_steps(gpu_lib, prec, cc):
    # 12 steps: the sort at tstep 10 makes the second captured graph
    p = case(prec=prec, cc=cc)
    eager = run(p, 21, 12, False)
    graph = run(p, 21, 12, True)
    assert_same(eager, graph)
    assert eager[2] == (0, 0)
    assert graph[2] == (11, 1)  # every step after the first was one graph launch


@pytest.mark.parametrize("gx,gz", [(0, 0), (1, 1)])
def test_graph_steps_with_temperature_tracers(gpu_lib, gx, gz):
    """Temperature tracers (tracer = 1, comp = 0): the stage's tracers_to_corners
    and T filter inside the captured step; uniform and stretched grids."""
    p = case(prec=0, cc=0, Ra=1e5, visT=100.0)
    p.comp, p.tracer, p.RaC[0] = 0, 1, 0.0
    p.gridX, p.gridZ, p.spaceX, p.spaceZ = gx, gz, 2.0, 1.0
    eager = run(p, 5, 6, False)
    graph = run(p, 5, 6, True)
    assert_same_fields(eager, graph, ("T", "SF", "rtr", "str", "Ttr"))
    assert graph[2] == (5, 1)


def assert_same_fields(a, b, keys):
    (ra, da, _), (rb, db, _) = a, b
    for (row_a, qa, dta), (row_b, qb, dtb) in zip(ra, rb):
        assert qa == qb and dta == dtb
        assert row_a == row_b
    for k in keys:
        assert np.array_equal(da[k], db[k]), k


def test_graph_steps_equal_eager_steps_at_512x128(gpu_lib):
    p = case(nx=512, nz=128, grids=5, prec=1, Ra=3e6, visT=3e3, tpc=6)
    assert_same(run(p, 5, 4, False), run(p, 5, 4, True))


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained weights")
def test_graph_steps_with_learned_start_and_direction(gpu_lib):
    p = case(nx=512, nz=128, grids=5, prec=1, Ra=3.3e6, visT=2.2e3, cc=4)
    p.learned_guess = 3
    eager = run(p, 777, 4, False, WEIGHTS)
    graph = run(p, 777, 4, True, WEIGHTS)
    assert_same(eager, graph)
    assert graph[2] == (3, 1)


def steps_until_error(p, seed, steps, graph):
    sim = Simulation(p)
    sim.upload(state.initial_state(p, seed=seed))
    if graph:
        sim.set_step_graph(True)
    out = []
    try:
        for _ in range(steps):
            out.append(sim.step()[1:])
        err = None
    except TracerError as e:
        err = e.status
    n = sim.step_graph_info()[0]
    sim.close()
    return out, err, n


def failing_case(seed=8, steps=10):
    """A case whose first (eager) step succeeds and a later one stops: a
    case whose tracers leave the box, else the smallest W-cycle cap that the
    first step meets."""
    cands = [case(prec=1, cc=0, Ra=1e5, visT=1e4), case(prec=0, cc=0), case(prec=1, cc=0), case(prec=1, cc=3)]
    for p in cands:
        out, err, _ = steps_until_error(p, seed, steps, False)
        if err is not None:
            if out:
                return p, out, err
            continue
        for cap in range(2, 400):
            q = p.copy()
            q.max_cycles = cap
            out, err, _ = steps_until_error(q, seed, steps, False)
            if err is None:
                break
            if out:
                return q, out, err
    return None


def test_graph_step_reports_the_eager_error(gpu_lib):
    found = failing_case()
    assert found is not None, "no case stops after its first step"
    p, out, err = found
    g_out, g_err, g_n = steps_until_error(p, 8, 10, True)
    print(f"stops after {len(out)} steps with status {err}")
    assert g_err == err
    assert g_out == out
    assert g_n == len(out)  # the failing step ran as a graph too


def test_ensemble_graph_steps_match_cases_alone(gpu_lib):
    from tracer_code_gb300.ensemble import Ensemble
    params = [case(256, 64, 4, 1, Ra=3e5), case(512, 128, 5, 1, Ra=2e6, visT=300.0),
              case(256, 64, 4, 0, Ra=1e6, visT=5e3, cc=0), case(512, 128, 5, 1, Ra=8e5, tpc=6)]
    seeds = [31, 32, 33, 34]
    ens = Ensemble(params, seeds=seeds, autotune=True)
    res = [ens.step() for _ in range(4)]
    graph_steps, eager_steps = ens.graph_info()
    states = [s.download() for s in ens.sims]
    tuning = ens.tuning
    ens.close()
    assert (graph_steps, eager_steps) == (3, 1)
    for i, p in enumerate(params):
        sim = Simulation(p)
        sim.set_launch_shapes(tuning[i])
        sim.upload(state.initial_state(p, seed=seeds[i]))
        for n in range(4):
            row, q, dt = sim.step()
            assert q == res[n][1][i] and dt == res[n][2][i]
            assert row == res[n][0][i]
        d = sim.download()
        for k in ("SF", "T", "rtr", "str"):
            assert np.array_equal(d[k], states[i][k]), (i, k)
        sim.close()
