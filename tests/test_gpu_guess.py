"""The learned initial guess inside the solver.

  - the recorder stores, per solve, the fields the solve started from and
    the converged streamfunction (FP32 images of the level-1 fields);
  - with any network attached (here an untrained one) every solve still
    meets the reference's tolerance: the solver starts from the network's
    guess only when its level-1 residual is smaller (and stops offering it
    after repeated rejections), and Nu/Vrms/mass after several steps agree
    with the run without the network to 1e-6 relative;
  - the committed trained network (tracer_code_gb300/weights), offered as
    the start, does not raise the W-cycle count of the mixed solver on a
    case whose physics it was not trained on (the counts are printed; the
    residual test keeps the plain start in practice);
  - the correction after every level-1 visit (cycle_correction 1: along
    psi's change over the last W-cycle; 2: also along the network's
    predicted change, the learned coarse-level correction; 3: over the
    changes of the last four W-cycles; 4: those and the network's change)
    and the residual-minimising learned start (learned_guess 3) keep every
    solve at the reference's tolerance, checked by the oracle's residual
    test, in FP64 and mixed precision, with no more W-cycles than without
    them;
  - on the 1024x256 workload the learned + mixed solver (windowed
    correction with the network's direction) takes strictly fewer W-cycles
    than the mixed solver alone and than the one-direction correction; the
    counts of the ablation without the network's direction are printed next
    to them (the share of the gain that the network itself brings).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from tracer_code_gb300 import Simulation, state
from tracer_code_gb300.abi import config_1024x256

pytestmark = pytest.mark.gpu

WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tracer_code_gb300", "weights",
                       "guess_512x128.npy")


def case(nx=256, nz=64, grids=4, prec=1, Ra=1e6, visT=1e3):
    p = config_1024x256()
    p.nx, p.nz, p.tpc, p.grids = nx, nz, 4, grids
    p.RaT = Ra
    p.RaC[0] = 0.6 * Ra
    p.visT = visT
    p.mg_zero_coarse = 1
    p.solver_precision = prec
    return p


def test_recorder_stores_solve_inputs_and_results(gpu_lib):
    from tracer_code_gb300 import learned
    p = case()
    sim = Simulation(p)
    sim.upload(state.initial_state(p, seed=4))
    sim.step()
    raw = torch.zeros((4, 3, p.nz, p.nx), dtype=torch.float32, device="cuda")
    sf = torch.zeros((4, p.nz, p.nx), dtype=torch.float32, device="cuda")
    learned.record_solves(sim, raw.data_ptr(), sf.data_ptr(), 4)
    sf_before = sim.download()["SF"]
    sim.multigrid()
    sf_after = sim.download()["SF"]
    assert learned.record_count(sim) == 1
    SP = 2
    prev = sf_before[SP:SP + p.nz, SP:SP + p.nx]  # nodes k = 0..nz-1, i = 0..nx-1
    new = sf_after[SP:SP + p.nz, SP:SP + p.nx]
    assert np.array_equal(raw[0, 2].cpu().numpy(), prev.astype(np.float32))
    assert np.array_equal(sf[0].cpu().numpy(), new.astype(np.float32))
    vis = sim.get("vis_grid", 1)[SP:SP + p.nz, SP:SP + p.nx]
    assert np.allclose(raw[0, 0].cpu().numpy(), np.log10(vis), rtol=1e-6, atol=1e-6)
    sim.step()  # four more solves, capacity 4 in total
    assert learned.record_count(sim) == 4
    sim.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_untrained_guess_keeps_the_solution(gpu_lib, prec):
    from tracer_code_gb300 import learned
    p = case(prec=prec)
    st = state.initial_state(p, seed=2)
    rows = []
    for use in (0, 1):
        q = p.copy()
        q.learned_guess = use
        sim = Simulation(q)
        net = learned.Net(1, p.nz, p.nx, seed=5)
        learned.attach(sim, net)
        sim.upload(st)
        rows.append([sim.step()[0] for _ in range(3)])
        if use:
            used, offered = learned.guess_stats(sim)
            # 12 solves; after 8 rejections in a row the guess is offered on
            # every 32nd solve only
            assert 8 <= offered <= 12 and used <= offered
        sim.close()
        net.close()
    for a, b in zip(rows[0], rows[1]):
        for key in ["Nu", "vrms"]:
            assert abs(a[key] - b[key]) <= 1e-6 * abs(a[key]), key
        assert abs(a["Cavg"][0] - b["Cavg"][0]) <= 1e-6 * abs(a["Cavg"][0])


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained weights")
def test_trained_guess_does_not_raise_cycle_count(gpu_lib):
    from tracer_code_gb300 import learned
    # physics inside the training ranges, seed and parameters not used in training
    p = case(nx=512, nz=128, grids=5, prec=1, Ra=3.3e6, visT=2.2e3)
    st = state.initial_state(p, seed=777)
    cycles = {}
    for use in (0, 1):
        q = p.copy()
        q.learned_guess = use
        sim = Simulation(q)
        net = learned.Net(1, p.nz, p.nx)
        net.load(WEIGHTS)
        learned.attach(sim, net)
        sim.upload(st)
        for _ in range(4):  # start-up transient, not counted
            sim.step()
        cycles[use] = sum(sim.step()[1] for _ in range(6))
        if use:
            cycles["used"], cycles["offered"] = learned.guess_stats(sim)
        sim.close()
        net.close()
    print(f"W-cycles over 6 steps: plain start {cycles[0]}, learned start {cycles[1]} "
          f"(guess used in {cycles['used']} of {cycles['offered']} solves)")
    assert cycles[1] <= cycles[0]


def _attach_trained(sim, p):
    from tracer_code_gb300 import learned
    net = learned.Net(1, p.nz, p.nx)
    if os.path.exists(WEIGHTS):
        net.load(WEIGHTS)
    learned.attach(sim, net)
    return net


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("cc,lg", [(1, 0), (2, 3), (3, 0), (4, 3)])
def test_cycle_correction_meets_tolerance(gpu_lib, prec, cc, lg):
    from oracle.pyoracle import Oracle
    from tests.cases import case_1024_like, fresh_state
    p = case_1024_like(nx=256, nz=64, grids=5, tpc=3, Ra=1e5, visT=1e4)
    p.mg_zero_coarse, p.solver_precision = 1, prec
    st = fresh_state(p, seed=2)
    cyc = {}
    for use in (0, 1):
        q = p.copy()
        q.cycle_correction, q.learned_guess = (cc, lg) if use else (0, 0)
        sim = Simulation(q)
        net = _attach_trained(sim, q) if use and cc in (2, 4) else None
        sim.upload(st)
        cyc[use] = sim.multigrid()
        sf = sim.download()["SF"]
        sim.close()
        if net:
            net.close()
    o = Oracle(p)
    o.upload(st)
    o.compute_viscosity(1)
    o.set("SF", sf)
    o.compute_rhs(1)
    ref = o.reference_residual(1)
    ratio = o.residual(1, from_sf=True) / ref
    o.close()
    print(f"precision {prec}, cycle_correction {cc}, learned_guess {lg}: W-cycles {cyc[0]} -> {cyc[1]}, "
          f"oracle residual ratio {ratio:.3e}")
    assert ratio <= p.tolerance
    assert cyc[1] <= cyc[0]


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained weights")
def test_learned_correction_on_workload(gpu_lib):
    p = config_1024x256()
    p.mg_zero_coarse, p.mg_coarse_matrix, p.solver_precision = 1, 1, 1
    st = state.initial_state(p, seed=1)
    runs = {}
    for name, cc, lg in (("mixed", 0, 0), ("one-direction correction", 1, 0),
                         ("windowed correction without network", 3, 0), ("learned + mixed", 4, 3)):
        q = p.copy()
        q.cycle_correction, q.learned_guess = cc, lg
        sim = Simulation(q)
        net = _attach_trained(sim, q) if cc in (2, 4) else None
        sim.upload(st)
        out = [sim.step() for _ in range(3)]
        runs[name] = ([c for _, c, _ in out], out[-1][0])
        sim.close()
        if net:
            net.close()
    for name, (c, _) in runs.items():
        print(f"1024x256 mixed, 3 steps, {name}: W-cycles {c} (total {sum(c)})")
    base, learned_run = runs["mixed"], runs["learned + mixed"]
    assert sum(learned_run[0]) < sum(base[0])
    assert sum(learned_run[0]) < sum(runs["one-direction correction"][0])
    for key in ("Nu", "vrms", "Tavg"):
        assert abs(learned_run[1][key] - base[1][key]) <= 1e-6 * abs(base[1][key]), key
