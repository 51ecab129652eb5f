"""tc_stats_noalloc: the stats.dat row from caller-owned device arrays,
computed without any device allocation by the library.

Callers that need it: a host that owns every device allocation itself (for
example an OpenACC or CUDA Fortran port of the reference keeping its arrays
in its own pool, or an application under a fixed device-memory budget) and
cannot let a library call cudaMalloc or create a tc_handle.

The test creates a case through the ordinary API, takes its fields in the
reference's layouts, places them in device memory that the TEST allocates,
and calls tc_stats_noalloc through the C ABI twice in a row; both rows must
equal the row of the existing entry point tc_stats (the parity tests accept
1e-6 relative for stats; the same kernels make these agree to 1e-12).  The
GPU's free memory must not change across the two calls (measured after one
warm-up call, which may load the library's kernels).  Three settings:
compositional tracers (comp = 1), temperature tracers only (comp = 0,
tracer = 1: the tracer-count columns are still filled, as in the reference),
and RaT = 0 passed for the same fields (the temperature columns are then 0,
as the reference leaves them unwritten).
The file name sorts last so a run that stops at the first failure has run
every other test first; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ["Tavg", "vrms", "Nu", "Nu_bot", "RaT_avg", "mobility", "strain_max", "q1", "q2", "q3", "q4"]
THERMAL = {"Tavg", "Nu", "Nu_bot", "RaT_avg", "q1", "q2", "q3", "q4"}


def _bind(L):
    vp = C.c_void_p
    from tracer_code_gb300.abi import StatsRow
    L.tc_stats_noalloc.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                   C.c_double, C.c_int32, vp, C.POINTER(StatsRow), vp]
    L.tc_stats_noalloc.restype = C.c_int


@pytest.mark.parametrize("setting", ["comp", "tracer_only", "isothermal"])
def test_stats_noalloc_matches_tc_stats(gpu_lib, setting):
    import torch
    from tracer_code_gb300 import Simulation
    from tracer_code_gb300.abi import StatsRow
    from tests.cases import case_1024_like, fresh_state

    L = gpu_lib
    _bind(L)
    p = case_1024_like()
    if setting == "tracer_only":
        p.comp, p.tracer, p.mg_zero_coarse = 0, 1, 1
    ntype = 1 if p.comp == 1 else 0
    sim = Simulation(p)
    sim.upload(fresh_state(p))
    sim.multigrid()
    sim.compute_velocities()
    ref = sim.stats()  # existing entry point; at tstep 0 it also fixes mass = Cavg
    nx, nz = sim.nx, sim.nz
    ds = 1.0 / nz
    kent = max(k for k in range(nz + 1) if ds * k <= p.dent)
    RaT = 0.0 if setting == "isothermal" else p.RaT

    host = {
        "T": sim.get("T"),
        "u": sim.get("u")[1:-1, 1:-1],
        "w": sim.get("w")[1:-1, 1:-1],
        "conduct": sim.get("conduct"),
        "vis": sim.get("vis_grid", 1),
        "nempty": sim.counts().sum(axis=2).astype(np.int32),
    }
    if ntype:
        host["Cnew"] = sim.get("Cnew", 0, 1)  # ntype = 1: (1:ntype, i, k) equals the plane
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in host.items()}
    cnew = dev["Cnew"].data_ptr() if ntype else None
    torch.cuda.synchronize()
    mass = (C.c_double * 4)(*ref["Cavg"])

    def call():
        row = StatsRow()
        st = L.tc_stats_noalloc(dev["T"].data_ptr(), dev["u"].data_ptr(), dev["w"].data_ptr(),
                                dev["conduct"].data_ptr(), dev["vis"].data_ptr(), cnew,
                                dev["nempty"].data_ptr(), nx, nz, ntype, p.aspect, RaT, kent, mass,
                                C.byref(row), None)
        return st, row.as_dict()

    assert call()[0] == 0  # warm-up: the first call may load the kernels
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for n in range(2):
        st, got = call()
        assert st == 0, (n, st)
        for key in KEYS:
            want = 0.0 if (RaT == 0.0 and key in THERMAL) else ref[key]
            assert abs(got[key] - want) <= 1e-12 * abs(want), (setting, n, key, got[key], want)
        if ntype:
            assert abs(got["Cavg"][0] - ref["Cavg"][0]) <= 1e-12 * abs(ref["Cavg"][0])
            assert abs(got["ent"][0] - ref["ent"][0]) <= 1e-12 * max(abs(ref["ent"][0]), 1e-300)
        for key in ("empty_cells", "tracer_min", "tracer_max"):
            assert got[key] == ref[key], (setting, n, key, got[key], ref[key])
        assert ref["tracer_max"] > 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0, "device memory changed across the calls"

    # sizes beyond the fixed buffer are refused without touching the GPU
    row = StatsRow()
    st = L.tc_stats_noalloc(dev["T"].data_ptr(), dev["u"].data_ptr(), dev["w"].data_ptr(),
                            dev["conduct"].data_ptr(), dev["vis"].data_ptr(), cnew,
                            dev["nempty"].data_ptr(), nx, 4097, ntype, p.aspect, RaT, kent, mass, C.byref(row), None)
    assert st == 12  # TC_ERR_TOO_LARGE
    sim.close()
