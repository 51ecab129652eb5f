"""Bounded device waits: a wait that runs out is reported as
TC_ERR_DEVICE_TIMEOUT and leaves the handle usable.  No GPU fault is
involved: a debug switch makes the kernel wait, with its bounded poll, for
a device word that nothing sets, before the kernel issues any copy or any
write to another CTA's shared memory; the poll runs out and the kernel
takes its ordinary timeout exit.

  - fused cluster visits of the multigrid (tc_debug_wait_test): the solve
    returns TC_ERR_DEVICE_TIMEOUT; with the switch off the same handle then
    solves exactly as a fresh handle does (same cycles, same SF);
  - the network's tcgen05 convolutions (tcnn_debug_wait_test, the
    convolution frees its tensor memory before returning): a solve that
    uses the network returns TC_ERR_DEVICE_TIMEOUT; with the switch off
    the next solve succeeds with the result of a handle that never failed.
"""
import os
import time

import numpy as np
import pytest

from tracer_code_gb300 import Simulation, TracerError
from tests.cases import case_1024_like, fresh_state

pytestmark = pytest.mark.gpu

TIMEOUT = 13  # TC_ERR_DEVICE_TIMEOUT
WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tracer_code_gb300", "weights",
                       "guess_512x128.npy")


def _solve(p, st, net=None):
    from tracer_code_gb300 import learned
    g = Simulation(p)
    if net is not None:
        learned.attach(g, net)
    g.upload(st)
    c = g.multigrid()
    sf = g.download()["SF"]
    g.close()
    return c, sf


@pytest.mark.parametrize("prec", [0, 1])
def test_cluster_visit_wait_runs_out_then_handle_solves(gpu_lib, prec):
    p = case_1024_like()
    p.mg_zero_coarse, p.solver_precision = 1, prec
    st = fresh_state(p, seed=8)
    c_ref, sf_ref = _solve(p, st)
    g = Simulation(p)
    g.upload(st)
    g.debug_wait_test(True)
    t0 = time.perf_counter()
    with pytest.raises(TracerError) as e:
        g.multigrid()
    waited = time.perf_counter() - t0
    assert e.value.status == TIMEOUT
    g.debug_wait_test(False)
    c = g.multigrid()
    sf = g.download()["SF"]
    g.close()
    print(f"precision {prec}: timed-out solve returned after {waited:.2f} s; then {c} cycles (fresh handle {c_ref})")
    assert c == c_ref
    assert np.abs(sf - sf_ref).max() <= 1e-12 * np.abs(sf_ref).max()


def test_network_conv_wait_runs_out_then_handle_solves(gpu_lib):
    from tracer_code_gb300 import learned
    p = case_1024_like(nx=256, nz=64, grids=5)
    p.mg_zero_coarse, p.solver_precision, p.learned_guess = 1, 1, 3
    st = fresh_state(p, seed=9)
    net = learned.Net(1, p.nz, p.nx)
    if os.path.exists(WEIGHTS):
        net.load(WEIGHTS)
    c_ref, sf_ref = _solve(p, st, net)
    g = Simulation(p)
    learned.attach(g, net)
    g.upload(st)
    net.debug_wait_test(True)
    with pytest.raises(TracerError) as e:
        g.multigrid()
    assert e.value.status == TIMEOUT
    net.debug_wait_test(False)
    c = g.multigrid()
    sf = g.download()["SF"]
    g.close()
    net.close()
    print(f"network timed out, then {c} cycles (handle that never failed: {c_ref})")
    assert c == c_ref
    assert np.abs(sf - sf_ref).max() <= 1e-12 * np.abs(sf_ref).max()
