"""GB300 (sm_103a) hot path of seantrim/tracer_code behind a C ABI.

``Simulation`` is the Python mirror of include/tracer_gpu.h: the methods
carry the names of the reference subroutines they replace (multigrid,
compute_velocities, stats, energy_time, tracers_to_corners) and raise
``TracerError`` where the reference would ``stop``.  The library is the
in-tree ``libtracer_gpu.so``; there is no CPU fallback: without the library
or without a GPU every call fails.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from .abi import (Info, Params, StatsRow, TracerError, config_1024x256, config_2048x512, config_plain_128,
                  default_params, scaled_config)
from . import restart, state, textio

__all__ = ["Simulation", "Params", "TracerError", "default_params", "config_plain_128", "config_1024x256",
           "config_2048x512", "scaled_config", "state", "restart", "textio", "load_library", "library_path"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libtracer_gpu.so")
_lock = threading.Lock()
_lib = None

EXPORTS = [
    "tc_default_params", "tc_abi_sizes", "tc_create", "tc_destroy", "tc_get_info", "tc_set_stream",
    "tc_upload_state", "tc_download_state", "tc_set_clock", "tc_multigrid", "tc_compute_velocities", "tc_stats",
    "tc_energy_time", "tc_step", "tc_download_velocities", "tc_tracers_to_corners", "tc_download_counts",
    "tc_last_error", "tc_debug_field", "tc_step_host", "tc_time_sweep", "tc_time_visit", "tc_time_subcycle", "tc_debug_wait_test", "tc_debug_sweep_fields", "tc_kernel_launches", "tc_autotune", "tc_ensemble_step",
    "tc_set_launch_shapes", "tc_tracer_order", "tc_compute_strain_rate_invariant", "tc_compute_viscosity",
    "tc_get_params", "tc_restart_write", "tc_restart_read", "tc_restart_tracers_write", "tc_restart_tracers_read",
    "tc_restart_grid", "tc_write_restart", "tc_read_restart", "tc_format_g", "tc_format_stats_line",
    "tc_format_vis_line", "tc_write_snapshot", "tc_upload_state_ex", "tc_download_tracer_temperature",
    "tc_equalize_row", "tc_format_equalize_line", "tc_set_step_graph", "tc_step_graph_info",
    "tc_ensemble_create", "tc_ensemble_run", "tc_ensemble_info", "tc_ensemble_destroy", "tc_grid_coordinates",
    "tc_grid_metrics",
]


def library_path() -> str:
    return _LIB_PATH


def load_library(build_if_missing: bool = False):
    """Loads libtracer_gpu.so (raises if it is missing: no fallback)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(_LIB_PATH):
            if build_if_missing:
                from .build import build
                build()
            else:
                raise RuntimeError(f"{_LIB_PATH} is missing: run `python -m tracer_code_gb300.build` "
                                   "(there is no CPU fallback)")
        L = C.CDLL(_LIB_PATH)
        vp = C.c_void_p
        L.tc_default_params.argtypes = [C.POINTER(Params)]
        L.tc_default_params.restype = None
        L.tc_abi_sizes.argtypes = [C.POINTER(C.c_int32)]
        L.tc_abi_sizes.restype = None
        L.tc_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
        L.tc_destroy.argtypes = [vp]
        L.tc_get_info.argtypes = [vp, C.POINTER(Info)]
        L.tc_set_stream.argtypes = [vp, vp]
        L.tc_upload_state.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_int64]
        L.tc_download_state.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.tc_upload_state_ex.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, C.c_int64]
        L.tc_download_tracer_temperature.argtypes = [vp, vp]
        L.tc_set_clock.argtypes = [vp, C.c_int32, C.c_double]
        L.tc_multigrid.argtypes = [vp, C.POINTER(C.c_int32)]
        L.tc_compute_velocities.argtypes = [vp]
        L.tc_stats.argtypes = [vp, C.POINTER(StatsRow)]
        L.tc_energy_time.argtypes = [vp, C.POINTER(C.c_double)]
        L.tc_step.argtypes = [vp, C.POINTER(StatsRow), C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.tc_download_velocities.argtypes = [vp, vp, vp]
        L.tc_tracers_to_corners.argtypes = [vp, vp, vp]
        L.tc_download_counts.argtypes = [vp, vp]
        L.tc_debug_field.argtypes = [vp, C.c_char_p, C.c_int32, C.c_int32, vp]
        L.tc_step_host.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_int64, C.POINTER(StatsRow),
                                   C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.tc_time_sweep.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(C.c_double)]
        L.tc_time_visit.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(C.c_double)]
        L.tc_time_subcycle.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(C.c_double)]
        L.tc_debug_wait_test.argtypes = [vp, C.c_int32]
        L.tc_debug_sweep_fields.argtypes = [vp, C.c_int32]
        L.tc_autotune.argtypes = [vp, vp]
        L.tc_set_launch_shapes.argtypes = [vp, vp]
        L.tc_tracer_order.argtypes = [vp, vp]
        L.tc_compute_strain_rate_invariant.argtypes = [vp]
        L.tc_compute_viscosity.argtypes = [vp, C.c_int32]
        L.tc_get_params.argtypes = [vp, C.POINTER(Params)]
        i32, cs = C.c_int32, C.c_char_p
        L.tc_restart_write.argtypes = [cs, i32, i32, i32, i32, vp, vp, vp, vp, vp]
        L.tc_restart_read.argtypes = [cs, i32, i32, i32, i32, vp, vp, vp, vp, vp]
        L.tc_restart_tracers_write.argtypes = [cs, C.c_int64, vp, vp, vp, vp]
        L.tc_restart_tracers_read.argtypes = [cs, C.c_int64, vp, vp, vp, vp]
        L.tc_restart_grid.argtypes = [i32, i32, C.c_double, vp, vp]
        L.tc_restart_grid.restype = None
        L.tc_write_restart.argtypes = [vp, cs, cs]
        L.tc_read_restart.argtypes = [vp, cs, cs]
        L.tc_format_g.argtypes = [C.c_double, i32, i32, i32, C.c_char_p]
        L.tc_format_g.restype = i32
        L.tc_format_stats_line.argtypes = [C.POINTER(StatsRow), i32, i32, i32, C.c_double, C.c_char_p, i32]
        L.tc_format_vis_line.argtypes = [C.POINTER(StatsRow), i32, i32, C.c_double, C.c_char_p, i32]
        L.tc_write_snapshot.argtypes = [vp, cs]
        L.tc_equalize_row.argtypes = [vp, C.POINTER(C.c_int64), i32, C.POINTER(i32)]
        L.tc_format_equalize_line.argtypes = [C.c_double, C.POINTER(C.c_int64), i32, C.c_char_p, i32]
        L.tc_ensemble_step.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, vp, vp, vp, vp]
        L.tc_set_step_graph.argtypes = [vp, C.c_int32]
        L.tc_step_graph_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
        L.tc_ensemble_create.argtypes = [C.c_int32, C.POINTER(vp)]
        L.tc_ensemble_run.argtypes = [vp, C.POINTER(vp), C.c_int32, vp, vp, vp, vp]
        L.tc_ensemble_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.tc_ensemble_destroy.argtypes = [vp]
        L.tc_grid_coordinates.argtypes = [vp, vp, vp]
        L.tc_grid_metrics.argtypes = [C.POINTER(Params), vp, vp]
        L.tc_kernel_launches.argtypes = []
        L.tc_kernel_launches.restype = C.c_int64
        L.tc_last_error.argtypes = [vp]
        L.tc_last_error.restype = C.c_char_p
        for name in EXPORTS:
            fn = getattr(L, name)
            if fn.restype is C.c_int:  # tc_status
                fn.restype = C.c_int
        sizes = (C.c_int32 * 3)()
        L.tc_abi_sizes(sizes)
        if (sizes[0], sizes[1], sizes[2]) != (C.sizeof(Params), C.sizeof(StatsRow), C.sizeof(Info)):
            raise RuntimeError(f"ABI mismatch: C sizes {tuple(sizes)} vs ctypes "
                               f"{(C.sizeof(Params), C.sizeof(StatsRow), C.sizeof(Info))}")
        _lib = L
        return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Simulation:
    """One case on one GPU (a tc_handle)."""

    def __init__(self, params: Params, stream: int | None = None):
        self.L = load_library()
        self.params = params.copy()
        h = C.c_void_p()
        st = self.L.tc_create(C.byref(self.params), C.byref(h))
        if st:
            raise TracerError(st, "tc_create")
        self.h = h
        self.info = Info()
        self.L.tc_get_info(self.h, C.byref(self.info))
        if stream is not None:
            self._chk(self.L.tc_set_stream(self.h, C.c_void_p(stream)), "tc_set_stream")

    def close(self):
        if getattr(self, "h", None):
            self.L.tc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, st, where):
        if st:
            msg = self.L.tc_last_error(self.h) if getattr(self, "h", None) else b""
            raise TracerError(st, where, (msg or b"").decode(errors="replace"))

    @property
    def nx(self):
        return self.info.nx

    @property
    def nz(self):
        return self.info.nz

    @property
    def ntr(self):
        return self.info.ntr

    def field_shape(self):
        s = self.info.span
        return (self.nz + 1 + 2 * s, self.nx + 1 + 2 * s)

    def set_stream(self, stream: int):
        self._chk(self.L.tc_set_stream(self.h, C.c_void_p(stream)), "tc_set_stream")

    def upload(self, st: dict):
        T = np.ascontiguousarray(st["T"], dtype=np.float64)
        SF = np.ascontiguousarray(st["SF"], dtype=np.float64)
        if T.shape != self.field_shape() or SF.shape != self.field_shape():
            raise TracerError(1, "upload", f"fields must have shape {self.field_shape()}")
        Cn = st.get("Cnew")
        Cn = None if Cn is None else np.ascontiguousarray(Cn, dtype=np.float64)
        r = st.get("rtr"); s = st.get("str"); t = st.get("Ttype")
        r = None if r is None else np.ascontiguousarray(r, dtype=np.float64)
        s = None if s is None else np.ascontiguousarray(s, dtype=np.float64)
        t = None if t is None else np.ascontiguousarray(t, dtype=np.int32)
        n = 0 if r is None else r.size
        if self.params.tracer == 1:
            tt = np.ascontiguousarray(st["Ttr"], dtype=np.float64)
            self._chk(self.L.tc_upload_state_ex(self.h, _ptr(T), _ptr(Cn), _ptr(SF), _ptr(r), _ptr(s), _ptr(t),
                                                _ptr(tt), n), "upload")
            return
        self._chk(self.L.tc_upload_state(self.h, _ptr(T), _ptr(Cn), _ptr(SF), _ptr(r), _ptr(s), _ptr(t), n), "upload")

    def download(self) -> dict:
        shp = self.field_shape()
        T = np.empty(shp); SF = np.empty(shp)
        nt = self.params.ntype if self.params.comp == 1 else 0
        Cn = np.empty(shp + (nt,)) if nt else None
        r = s = t = None
        if self.params.comp == 1 or self.params.tracer == 1:
            r = np.empty(self.ntr); s = np.empty(self.ntr)
        if self.params.comp == 1:
            t = np.empty(self.ntr, dtype=np.int32)
        self._chk(self.L.tc_download_state(self.h, _ptr(T), _ptr(Cn), _ptr(SF), _ptr(r), _ptr(s), _ptr(t)),
                  "download")
        out = {"T": T, "SF": SF}
        if nt:
            out["Cnew"] = Cn
        if r is not None:
            out.update(rtr=r, str=s)
        if t is not None:
            out["Ttype"] = t
        if self.params.tracer == 1:
            tt = np.empty(self.ntr)
            self._chk(self.L.tc_download_tracer_temperature(self.h, _ptr(tt)), "download_tracer_temperature")
            out["Ttr"] = tt
        return out

    def set_clock(self, tstep: int, time: float):
        self._chk(self.L.tc_set_clock(self.h, tstep, time), "set_clock")

    def multigrid(self) -> int:
        q = C.c_int32(0)
        self._chk(self.L.tc_multigrid(self.h, C.byref(q)), "multigrid")
        return q.value

    def compute_velocities(self):
        self._chk(self.L.tc_compute_velocities(self.h), "compute_velocities")

    def stats(self) -> dict:
        row = StatsRow()
        self._chk(self.L.tc_stats(self.h, C.byref(row)), "stats")
        return row.as_dict()

    def energy_time(self) -> float:
        dt = C.c_double(0)
        self._chk(self.L.tc_energy_time(self.h, C.byref(dt)), "energy_time")
        return dt.value

    def step(self):
        row = StatsRow(); q = C.c_int32(0); dt = C.c_double(0)
        self._chk(self.L.tc_step(self.h, C.byref(row), C.byref(q), C.byref(dt)), "step")
        return row.as_dict(), q.value, dt.value

    def grid_coordinates(self):
        """(xg, zg): the handle's node coordinates, index i + 3 for i = -3..n+3."""
        xg = np.empty(self.nx + 7); zg = np.empty(self.nz + 7)
        self._chk(self.L.tc_grid_coordinates(self.h, _ptr(xg), _ptr(zg)), "grid_coordinates")
        return xg, zg

    def set_step_graph(self, on: bool = True) -> None:
        """From the next ready step on, each tc_step is one captured graph
        launch (tc_set_step_graph)."""
        self._chk(self.L.tc_set_step_graph(self.h, 1 if on else 0), "set_step_graph")

    def step_graph_info(self):
        """(steps run as one graph launch, state 0 off / 1 on / 2 refused)."""
        n = C.c_int64(0); st = C.c_int32(0)
        self._chk(self.L.tc_step_graph_info(self.h, C.byref(n), C.byref(st)), "step_graph_info")
        return n.value, st.value

    def step_host(self, st: dict):
        """tc_step_host on host arrays (pinned for end-to-end timing); st is
        updated in place and must hold the state the previous call returned."""
        row = StatsRow(); q = C.c_int32(0); dt = C.c_double(0)
        n = 0 if st.get("rtr") is None else st["rtr"].size
        self._chk(self.L.tc_step_host(self.h, _ptr(st["T"]), _ptr(st.get("Cnew")), _ptr(st["SF"]),
                                      _ptr(st.get("rtr")), _ptr(st.get("str")), _ptr(st.get("Ttype")), n,
                                      C.byref(row), C.byref(q), C.byref(dt)), "step_host")
        return row.as_dict(), q.value, dt.value

    def time_sweep(self, level: int = 1, nsweeps: int = 70) -> float:
        ms = C.c_double(0)
        self._chk(self.L.tc_time_sweep(self.h, level, nsweeps, C.byref(ms)), "time_sweep")
        return ms.value

    def autotune(self) -> list:
        """Runs tc_autotune; returns [(block_x, block_y, fused)] for levels 1..grids-1."""
        g = self.info.grids
        out = (C.c_int32 * (3 * max(g - 1, 1)))()
        self._chk(self.L.tc_autotune(self.h, out), "autotune")
        return [(out[3 * i], out[3 * i + 1], out[3 * i + 2]) for i in range(g - 1)]

    def compute_strain(self) -> None:
        self._chk(self.L.tc_compute_strain_rate_invariant(self.h), "compute_strain_rate_invariant")

    def compute_viscosity(self, level: int = 1) -> None:
        self._chk(self.L.tc_compute_viscosity(self.h, level), "compute_viscosity")

    def tracer_order(self):
        """perm[j] = reference index of the tracer in device storage slot j."""
        perm = np.empty(self.ntr, np.int32)
        self._chk(self.L.tc_tracer_order(self.h, perm.ctypes.data_as(C.c_void_p)), "tracer_order")
        return perm

    def set_launch_shapes(self, choices) -> None:
        """Applies [(block_x, block_y, visit)] per level 1..grids-1 (autotune()'s format)."""
        flat = [int(v) for c in choices for v in c]
        arr = (C.c_int32 * max(len(flat), 1))(*flat)
        self._chk(self.L.tc_set_launch_shapes(self.h, arr), "set_launch_shapes")

    def time_visit(self, level: int, reps: int = 20) -> float:
        ms = C.c_double(0)
        self._chk(self.L.tc_time_visit(self.h, level, reps, C.byref(ms)), "time_visit")
        return ms.value

    def time_subcycle(self, k: int, reps: int = 20) -> float:
        """ms per product with the bottom-of-cycle matrix of the pattern with k coarsest solves."""
        ms = C.c_double(0)
        self._chk(self.L.tc_time_subcycle(self.h, k, reps, C.byref(ms)), "time_subcycle")
        return ms.value

    def debug_wait_test(self, on: bool) -> None:
        """Timeout-path test: fused visits wait on a word nothing sets (tc_debug_wait_test)."""
        self._chk(self.L.tc_debug_wait_test(self.h, 1 if on else 0), "debug_wait_test")

    def debug_sweep_fields(self, fields: bool) -> None:
        """Level-1 FP32 sweep from the five viscosity fields (default) or from
        the 13 coefficient planes (tc_debug_sweep_fields)."""
        self._chk(self.L.tc_debug_sweep_fields(self.h, 1 if fields else 0), "debug_sweep_fields")

    @staticmethod
    def kernel_launches() -> int:
        return int(load_library().tc_kernel_launches())

    def velocities(self):
        shp = (self.nz + 3, self.nx + 3)
        u = np.empty(shp); w = np.empty(shp)
        self._chk(self.L.tc_download_velocities(self.h, _ptr(u), _ptr(w)), "download_velocities")
        return u, w

    def tracers_to_corners(self, r, s):
        r = np.ascontiguousarray(r, np.float64); s = np.ascontiguousarray(s, np.float64)
        self._chk(self.L.tc_tracers_to_corners(self.h, _ptr(r), _ptr(s)), "tracers_to_corners")

    def get(self, name: str, level: int = 1, type_: int = 0) -> np.ndarray:
        """Diagnostic copy of an internal field on the level's ghost-padded box."""
        a = self.info.nx_grid[level - 1] if level >= 1 else self.nx
        b = self.info.nz_grid[level - 1] if level >= 1 else self.nz
        s = self.info.span
        out = np.empty((b + 1 + 2 * s, a + 1 + 2 * s))
        self._chk(self.L.tc_debug_field(self.h, name.encode(), level, type_, _ptr(out)), f"debug_field {name}")
        return out

    def counts(self) -> np.ndarray:
        nt = (self.params.ntype if self.params.comp == 1 else 0) + 1
        out = np.empty(self.field_shape() + (nt,), dtype=np.int32)
        self._chk(self.L.tc_download_counts(self.h, _ptr(out)), "download_counts")
        return out

    def write_restart(self, trestart: str, tracers: str | None = None) -> None:
        """print_restart (main.f90:301-330): Trestart and, for comp = 1, restart_tracers."""
        self._chk(self.L.tc_write_restart(self.h, os.fsencode(trestart),
                                          None if tracers is None else os.fsencode(tracers)), "write_restart")

    def read_restart(self, trestart: str, tracers: str | None = None) -> None:
        """build_grid's restart branch (grid.f90:55-96) followed by tc_upload_state."""
        self._chk(self.L.tc_read_restart(self.h, os.fsencode(trestart),
                                         None if tracers is None else os.fsencode(tracers)), "read_restart")

    def write_snapshot(self, path: str) -> None:
        """snapshots (main.f90:237-270): the T1xxxx text file of the current state (call after stats)."""
        self._chk(self.L.tc_write_snapshot(self.h, os.fsencode(path)), "write_snapshot")

    def equalize_row(self) -> list:
        """The equalize.dat values of the last tracer repositioning (tc_equalize_row); [] if none."""
        out = (C.c_int64 * 64)(); n = C.c_int32(0)
        self._chk(self.L.tc_equalize_row(self.h, out, 64, C.byref(n)), "equalize_row")
        return [int(out[q]) for q in range(n.value)]
