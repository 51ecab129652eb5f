"""ctypes mirror of include/tracer_gpu.h (structs, defaults, configurations).

The field order of ``Params`` must match ``tc_params`` exactly; the C side
checks ``sizeof`` through ``tc_params_size`` when the library is loaded.
"""
from __future__ import annotations

import ctypes as C
import math

TC_MAX_TYPES = 4

STATUS = {
    0: "TC_OK",
    1: "TC_ERR_ARG",
    2: "TC_ERR_UNSUPPORTED",
    3: "TC_ERR_MG_CYCLES",
    4: "TC_ERR_MG_RESIDUAL",
    5: "TC_ERR_TRACER_OUTSIDE",
    6: "TC_ERR_RK2_STABILITY",
    7: "TC_ERR_LOOP_CAP",
    8: "TC_ERR_CUDA",
    9: "TC_ERR_ALLOC",
    10: "TC_ERR_STATE",
    11: "TC_ERR_SINGULAR",
    12: "TC_ERR_TOO_LARGE",
    13: "TC_ERR_DEVICE_TIMEOUT",
    14: "TC_ERR_EQUALIZE",
}

# Reference `stop` messages that each status replaces.
STOP_MESSAGES = {
    3: "Multigrid Convergence Problem: Too Many Multigrid Cycles Needed",
    4: "Multigrid Convergence Problem: Abnormally High Residual Detected -- stopping",
    5: "Tracer advected outside of domain - stopping",
    6: "Advective Eigenvalues Exceed Diffusive Eigenvalues -- this does not work for RK2",
    14: "Error: # of donor tracers found inconsistent with nfree value",
}


class TracerError(RuntimeError):
    """A non-zero tc_status, i.e. one of the reference's `stop` sites."""

    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        name = STATUS.get(status, f"status {status}")
        msg = f"{where}: {name}"
        if status in STOP_MESSAGES:
            msg += f" ({STOP_MESSAGES[status]})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


_D4 = C.c_double * TC_MAX_TYPES
_I4 = C.c_int32 * TC_MAX_TYPES


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("nz", C.c_int32), ("aspect", C.c_double), ("order", C.c_int32),
        ("gridX", C.c_int32), ("gridZ", C.c_int32), ("spaceX", C.c_double), ("spaceZ", C.c_double),
        ("thickness", C.c_double), ("nbound", C.c_int32),
        ("non_Newtonian", C.c_int32), ("iterate_order", C.c_int32), ("tolerance", C.c_double),
        ("Nmulti", C.c_int32), ("mingrid", C.c_int32), ("grids", C.c_int32), ("eig_ratio", C.c_double),
        ("vis_iter", C.c_int32), ("max_cycles", C.c_int32),
        ("torder", C.c_int32), ("courant", C.c_double), ("courantT", C.c_double), ("courantC", C.c_double),
        ("courant_stream", C.c_double), ("RK_update", C.c_int32), ("dt_manual", C.c_double),
        ("comp", C.c_int32), ("ntype", C.c_int32), ("tpc", C.c_int32), ("dist_factor", C.c_double),
        ("Tbot", C.c_int32), ("Vbc", C.c_int32), ("dlayer", C.c_double), ("dent", C.c_double),
        ("RaT", C.c_double), ("RaC", _D4), ("H", C.c_double), ("conduct_factor", _D4), ("Htype", _D4),
        ("eig_ratio_min", C.c_double), ("ivis", C.c_int32), ("visP", C.c_double), ("visT", C.c_double),
        ("delta_visT", C.c_double), ("yield_", C.c_double), ("yield_gradient", C.c_double),
        ("yield_depth", C.c_double), ("visC", _D4), ("delta_visC", _D4),
        ("mg_zero_coarse", C.c_int32), ("solver_precision", C.c_int32), ("learned_guess", C.c_int32), ("learned_smooth", C.c_int32),
        ("tracer_sort_interval", C.c_int32), ("tracer", C.c_int32), ("equalize", C.c_int32),
        ("equalize_threads", C.c_int32), ("mg_coarse_matrix", C.c_int32), ("cycle_correction", C.c_int32),
    ]

    def copy(self) -> "Params":
        q = Params()
        C.memmove(C.byref(q), C.byref(self), C.sizeof(Params))
        return q


class StatsRow(C.Structure):
    _fields_ = [
        ("time", C.c_double), ("Tavg", C.c_double), ("vrms", C.c_double), ("Nu", C.c_double),
        ("Nu_bot", C.c_double), ("RaT_avg", C.c_double), ("mobility", C.c_double), ("strain_max", C.c_double),
        ("q1", C.c_double), ("q2", C.c_double), ("q3", C.c_double), ("q4", C.c_double),
        ("empty_cells", C.c_int32), ("tracer_min", C.c_int32), ("tracer_max", C.c_int32), ("tstep", C.c_int32),
        ("Cavg", _D4), ("ent", _D4), ("n_eta", C.c_int32), ("n_temp", C.c_int32), ("n_comp", _I4),
        ("eig_fine", C.c_double),
    ]

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if hasattr(v, "__len__"):
                v = list(v)
            d[name] = v
        return d


class Info(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("nz", C.c_int32), ("span", C.c_int32), ("span_interp", C.c_int32),
        ("grids", C.c_int32), ("nsteps", C.c_int32), ("ntr", C.c_int64), ("ngrid_coarse", C.c_int32),
        ("kl", C.c_int32), ("ku", C.c_int32), ("nx_grid", C.c_int32 * 8), ("nz_grid", C.c_int32 * 8),
        ("dr", C.c_double), ("ds", C.c_double),
    ]


def default_params() -> Params:
    """The shipped main.f90:8-116 inputs, switched to the implemented path:
    compositional tracers (comp=1, ntype=1, tracer=0, equalize=0),
    Newtonian viscosity (non_Newtonian=0, ivis=2) and RK4 (torder=4; RK2 is
    only valid with temperature tracers, main.f90:37).  Mirrors the C
    function tc_default_params."""
    p = Params()
    p.nx, p.nz, p.aspect, p.order = 200, 200, 1.0, 2
    p.gridX, p.gridZ, p.spaceX, p.spaceZ, p.thickness, p.nbound = 0, 0, 1.0, 1.0, 0.1, 8
    p.non_Newtonian, p.iterate_order, p.tolerance = 0, 1, 1.0e-3
    p.Nmulti, p.mingrid, p.grids, p.eig_ratio, p.vis_iter, p.max_cycles = 70, 4, 2, 4.0, 12, 1000
    p.torder, p.courant, p.courantT, p.courantC, p.courant_stream = 4, 0.99, 0.99, 0.99, 0.99
    p.RK_update, p.dt_manual = 1, 0.5
    p.comp, p.ntype, p.tpc, p.dist_factor = 1, 1, 30, 1.0e-4
    p.Tbot, p.Vbc, p.dlayer, p.dent = 0, 0, 0.1, 0.1
    p.RaT = 1.0e3 / 3.0
    p.H = 0.0
    for t in range(TC_MAX_TYPES):
        p.RaC[t] = 0.0
        p.conduct_factor[t] = 1.0
        p.Htype[t] = 0.0
        p.visC[t] = 1.0
        p.delta_visC[t] = 2.0
    p.eig_ratio_min, p.ivis, p.visP, p.visT, p.delta_visT = 4.0, 2, 1.0, 3.0e4, 100.0
    p.yield_, p.yield_gradient, p.yield_depth = 15.0, 0.0, 0.1
    p.tracer_sort_interval = 10
    return p


def config_plain_128(tpc: int = 20) -> Params:
    """Plain FP64 case that runs on CPU with the reference: aspect 1,
    128x128 cells, Ra=1e5, B=0.5, isoviscous, dense layer z<0.2, 20 tracers
    per cell, multigrid to 1e-8."""
    p = default_params()
    p.nx, p.nz, p.aspect = 128, 128, 1.0
    p.grids, p.tolerance = 6, 1.0e-8
    p.tpc = tpc
    p.RaT = 1.0e5
    p.RaC[0] = 0.5 * 1.0e5
    p.ivis = 0
    p.visT = 1.0
    p.dlayer = 0.2
    return p


def config_1024x256(tpc: int = 25) -> Params:
    """GPU drop-in case: aspect 4, 1024x256 cells, 25 tracers per cell
    (6,585,625 tracers), Ra=1e7, B=0.8, dense layer z<0.1,
    eta = exp(-ln(1e4) T) x 10 in enriched material (ivis=2, visC=1/10)."""
    p = default_params()
    p.nx, p.nz, p.aspect = 1024, 256, 4.0
    p.grids, p.tolerance = 6, 1.0e-8
    p.tpc = tpc
    p.RaT = 1.0e7
    p.RaC[0] = 0.8 * 1.0e7
    p.ivis = 2
    p.visT = 1.0e4
    p.visC[0] = 0.1
    p.dlayer = 0.1
    return p


def config_2048x512(tpc: int = 40) -> Params:
    """Large case: aspect 4, 2048x512 cells, 40 tracers per cell
    (42,045,480 tracers), Ra=1e8, B=1.0, contrast 1e6 (T) x 30 (C)."""
    p = default_params()
    p.nx, p.nz, p.aspect = 2048, 512, 4.0
    p.grids, p.tolerance = 6, 1.0e-8
    p.tpc = tpc
    p.RaT = 1.0e8
    p.RaC[0] = 1.0 * 1.0e8
    p.ivis = 2
    p.visT = 1.0e6
    p.visC[0] = 1.0 / 30.0
    p.dlayer = 0.1
    return p


def scaled_config(base: Params, nx: int, nz: int, tpc: int | None = None) -> Params:
    """Same physics on another grid (used for parity cases small enough for
    the oracle)."""
    p = base.copy()
    p.nx, p.nz = nx, nz
    if tpc is not None:
        p.tpc = tpc
    return p


def params_summary(p: Params) -> dict:
    return {
        "nx": p.nx, "nz": p.nz, "aspect": p.aspect, "tpc": p.tpc, "RaT": p.RaT, "RaC": p.RaC[0],
        "ivis": p.ivis, "visT": p.visT, "visC": p.visC[0], "grids": p.grids, "Nmulti": p.Nmulti,
        "tolerance": p.tolerance, "torder": p.torder,
    }


def _check() -> None:
    assert math.isclose(default_params().RaT, 1000.0 / 3.0)


_check()
