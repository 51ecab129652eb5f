"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only the tests, ``__graft_entry__.smoke()`` (to compare against) and the CPU
baseline leg of ``bench.py`` may import this module.  It exposes the same
methods as ``tracer_code_gb300.Simulation`` so a parity test runs both on the
same inputs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

from tracer_code_gb300.abi import Info, Params, StatsRow, TracerError

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compiles oracle.cpp with the recipe in oracle/Makefile."""
    src = os.path.join(_HERE, "oracle.cpp")
    hdr = os.path.join(os.path.dirname(_HERE), "include", "tracer_gpu.h")
    stale = (not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(src), os.path.getmtime(hdr)))
    if force or stale:
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "liboracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            vp = C.c_void_p
            dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
            ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
            L.tco_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
            L.tco_destroy.argtypes = [vp]
            L.tco_get_info.argtypes = [vp, C.POINTER(Info)]
            L.tco_upload_state.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_int64]
            L.tco_download_state.argtypes = [vp, vp, vp, vp, vp, vp, vp]
            L.tco_upload_state_ex.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, C.c_int64]
            L.tco_download_ttr.argtypes = [vp, vp]
            L.tco_equalize_row.argtypes = [vp, C.POINTER(C.c_int64), C.c_int32, C.POINTER(C.c_int32)]
            L.tco_set_clock.argtypes = [vp, C.c_int32, C.c_double]
            L.tco_multigrid.argtypes = [vp, C.POINTER(C.c_int32)]
            L.tco_set_max_cycles.argtypes = [vp, C.c_int32]
            L.tco_residual_trace.argtypes = [vp, dp, C.c_int32]
            L.tco_residual_trace.restype = C.c_int
            L.tco_compute_velocities.argtypes = [vp]
            L.tco_stats.argtypes = [vp, C.POINTER(StatsRow)]
            L.tco_energy_time.argtypes = [vp, C.POINTER(C.c_double)]
            L.tco_step.argtypes = [vp, C.POINTER(StatsRow), C.POINTER(C.c_int32), C.POINTER(C.c_double)]
            L.tco_tracers_to_corners.argtypes = [vp, dp, dp]
            L.tco_download_counts.argtypes = [vp, ip]
            L.tco_download_nempty.argtypes = [vp, ip]
            L.tco_field_shape.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_int32)]
            L.tco_get_field.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, dp]
            L.tco_set_field.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, dp]
            L.tco_compute_strain.argtypes = [vp]
            L.tco_compute_viscosity.argtypes = [vp, C.c_int]
            L.tco_compute_rhs.argtypes = [vp, C.c_int]
            L.tco_reference_residual.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
            L.tco_residual.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
            L.tco_local_time_steps.argtypes = [vp, C.c_int]
            L.tco_smoother_time_T.argtypes = [vp]
            L.tco_scalars.argtypes = [vp, dp]
            L.tco_eig_bases.argtypes = [vp, dp]
            L.tco_coordinates.argtypes = [vp, dp, dp]
            L.tco_metrics.argtypes = [vp, dp, dp]
            L.tco_fd_coefficients.argtypes = [vp, dp]
            L.tco_coarse_matrix.argtypes = [vp, dp, dp]
            L.tco_set_threads.argtypes = [C.c_int]
            L.tco_get_tracers.argtypes = [vp, C.c_int, dp]
            _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """CPU restatement of the reference; same interface as tracer_code_gb300.Simulation."""

    def __init__(self, params: Params, threads: int | None = None):
        self.L = lib()
        if threads is not None:
            self.L.tco_set_threads(int(threads))
        self.params = params.copy()
        h = C.c_void_p()
        st = self.L.tco_create(C.byref(self.params), C.byref(h))
        if st:
            raise TracerError(st, "tco_create")
        self.h = h
        self.info = Info()
        self.L.tco_get_info(self.h, C.byref(self.info))

    def close(self):
        if getattr(self, "h", None):
            self.L.tco_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st, where):
        if st:
            raise TracerError(st, where)

    # geometry helpers
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

    def upload(self, state: dict):
        T = np.ascontiguousarray(state["T"], dtype=np.float64)
        SF = np.ascontiguousarray(state["SF"], dtype=np.float64)
        Cn = state.get("Cnew")
        Cn = None if Cn is None else np.ascontiguousarray(Cn, dtype=np.float64)
        r = state.get("rtr"); s = state.get("str"); t = state.get("Ttype")
        r = None if r is None else np.ascontiguousarray(r, dtype=np.float64)
        s = None if s is None else np.ascontiguousarray(s, dtype=np.float64)
        t = None if t is None else np.ascontiguousarray(t, dtype=np.int32)
        n = 0 if r is None else r.size
        if self.params.tracer == 1:
            tt = np.ascontiguousarray(state["Ttr"], dtype=np.float64)
            self._chk(self.L.tco_upload_state_ex(self.h, _ptr(T), _ptr(Cn), _ptr(SF), _ptr(r), _ptr(s), _ptr(t),
                                                 _ptr(tt), n), "upload")
            return
        self._chk(self.L.tco_upload_state(self.h, _ptr(T), _ptr(Cn), _ptr(SF), _ptr(r), _ptr(s), _ptr(t), n), "upload")

    def download(self) -> dict:
        shp = self.field_shape()
        T = np.empty(shp); SF = np.empty(shp)
        nt = self.params.ntype if self.params.comp == 1 else 0
        Cn = np.empty(shp + (nt,)) if nt else None
        out = {"T": T, "SF": SF}
        r = s = t = None
        if self.params.comp == 1 or self.params.tracer == 1:
            r = np.empty(self.ntr); s = np.empty(self.ntr); t = np.empty(self.ntr, dtype=np.int32)
        self.L.tco_download_state(self.h, _ptr(T), _ptr(Cn), _ptr(SF), _ptr(r), _ptr(s), _ptr(t))
        if nt:
            out["Cnew"] = Cn
        if r is not None:
            out.update(rtr=r, str=s)
            if self.params.comp == 1:
                out["Ttype"] = t
        if self.params.tracer == 1:
            tt = np.empty(self.ntr)
            self._chk(self.L.tco_download_ttr(self.h, _ptr(tt)), "download_ttr")
            out["Ttr"] = tt
        return out

    def set_clock(self, tstep: int, time: float):
        self.L.tco_set_clock(self.h, tstep, time)

    def multigrid(self) -> int:
        q = C.c_int32(0)
        self._chk(self.L.tco_multigrid(self.h, C.byref(q)), "multigrid")
        return q.value

    def set_max_cycles(self, n: int):
        self._chk(self.L.tco_set_max_cycles(self.h, n), "set_max_cycles")

    def residual_trace(self) -> np.ndarray:
        """Level-1 residual ratio after each W-cycle of the last multigrid call."""
        buf = np.zeros(4096)
        n = self.L.tco_residual_trace(self.h, buf, buf.size)
        return buf[:min(n, buf.size)].copy()

    def compute_velocities(self):
        self.L.tco_compute_velocities(self.h)

    def stats(self) -> dict:
        row = StatsRow()
        self.L.tco_stats(self.h, C.byref(row))
        return row.as_dict()

    def energy_time(self) -> float:
        dt = C.c_double(0)
        self._chk(self.L.tco_energy_time(self.h, C.byref(dt)), "energy_time")
        return dt.value

    def step(self):
        row = StatsRow(); q = C.c_int32(0); dt = C.c_double(0)
        self._chk(self.L.tco_step(self.h, C.byref(row), C.byref(q), C.byref(dt)), "step")
        return row.as_dict(), q.value, dt.value

    def tracers_to_corners(self, r, s):
        self._chk(self.L.tco_tracers_to_corners(self.h, np.ascontiguousarray(r, np.float64),
                                                np.ascontiguousarray(s, np.float64)), "tracers_to_corners")

    def counts(self) -> np.ndarray:
        nt = (self.params.ntype if self.params.comp == 1 else 0) + 1
        shp = self.field_shape()
        out = np.empty(shp + (nt,), dtype=np.int32)
        self.L.tco_download_counts(self.h, out.reshape(-1))
        return out

    def nempty(self) -> np.ndarray:
        out = np.empty(self.field_shape(), dtype=np.int32)
        self.L.tco_download_nempty(self.h, out.reshape(-1))
        return out

    def velocities(self):
        return self.get("u"), self.get("w")

    # --- oracle-only hooks ---
    def shape(self, name, level=0, type_=0):
        b = (C.c_int32 * 4)()
        self._chk(self.L.tco_field_shape(self.h, name.encode(), level, type_, b), f"shape {name}")
        return tuple(b)

    def get(self, name, level=0, type_=0) -> np.ndarray:
        i0, i1, k0, k1 = self.shape(name, level, type_)
        out = np.empty((k1 - k0 + 1, i1 - i0 + 1))
        self._chk(self.L.tco_get_field(self.h, name.encode(), level, type_, out.reshape(-1)), f"get {name}")
        return out

    def set(self, name, arr, level=0, type_=0):
        i0, i1, k0, k1 = self.shape(name, level, type_)
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(k1 - k0 + 1, i1 - i0 + 1)
        self._chk(self.L.tco_set_field(self.h, name.encode(), level, type_, a.reshape(-1)), f"set {name}")

    def compute_strain(self):
        self.L.tco_compute_strain(self.h)

    def compute_viscosity(self, level: int):
        self._chk(self.L.tco_compute_viscosity(self.h, level), "compute_viscosity")

    def compute_rhs(self, level: int):
        self.L.tco_compute_rhs(self.h, level)

    def reference_residual(self, level: int) -> float:
        v = C.c_double(0)
        self.L.tco_reference_residual(self.h, level, C.byref(v))
        return v.value

    def residual(self, level: int, from_sf: bool = True) -> float:
        v = C.c_double(0)
        self._chk(self.L.tco_residual(self.h, level, int(from_sf), C.byref(v)), "residual")
        return v.value

    def local_time_steps(self, level: int):
        self.L.tco_local_time_steps(self.h, level)

    def smoother_time_T(self):
        self._chk(self.L.tco_smoother_time_T(self.h), "smoother_time_T")

    def scalars(self) -> dict:
        out = np.empty(8)
        self.L.tco_scalars(self.h, out)
        keys = ["eig_fine", "n_eta", "n_temp", "dt", "delta_T", "res_ref1", "residual_mag1", "cycles"]
        return dict(zip(keys, out.tolist()))

    def coordinates(self):
        """(xg, zg): build_grid's node coordinates, index i + 3 for i = -3..n+3."""
        xg = np.empty(self.nx + 7); zg = np.empty(self.nz + 7)
        self.L.tco_coordinates(self.h, xg, zg)
        return xg, zg

    def metrics(self):
        """(x5, z5): xr, xrr, xrrr, xrrrr, DERxr (and z) as rows over -3..n+3."""
        x5 = np.empty(5 * (self.nx + 7)); z5 = np.empty(5 * (self.nz + 7))
        self.L.tco_metrics(self.h, x5, z5)
        return x5.reshape(5, -1), z5.reshape(5, -1)

    def eig_bases(self) -> dict:
        out = np.empty(12)
        self.L.tco_eig_bases(self.h, out)
        keys = ["Tr", "Trr", "Trrr", "Trrrr", "Ts", "Tss", "Tsss", "Tssss", "Trs", "Trrss", "Trss", "Trrs"]
        return dict(zip(keys, out.tolist()))

    def fd_coefficients(self) -> dict:
        out = np.empty(64)
        self.L.tco_fd_coefficients(self.h, out)
        s = self.info.span
        n = 2 * s + 1
        si = self.info.span_interp
        m = 2 * si + 1
        d = {"D1": out[0:n], "D2": out[n:2 * n], "D3": out[2 * n:3 * n], "D4": out[3 * n:4 * n]}
        dn = self.params.order
        for j in range(dn):
            d[f"D{j + 1}_interp"] = out[4 * n + j * m: 4 * n + (j + 1) * m]
        return d

    def tracers(self, which: str) -> np.ndarray:
        names = ["rtr", "str", "rtr0", "str0", "rtr1", "str1", "rtr2", "str2"]
        out = np.empty(self.ntr)
        self._chk(self.L.tco_get_tracers(self.h, names.index(which), out), "tracers")
        return out

    def coarse_matrix(self):
        ldab = 2 * self.info.kl + self.info.ku + 1
        n = self.info.ngrid_coarse
        band = np.empty(ldab * n)
        rowb = np.empty(n)
        self.L.tco_coarse_matrix(self.h, band, rowb)
        return band.reshape(n, ldab), rowb

    def equalize_row(self) -> list:
        out = (C.c_int64 * 64)(); n = C.c_int32(0)
        self._chk(self.L.tco_equalize_row(self.h, out, 64, C.byref(n)), "equalize_row")
        return [int(out[q]) for q in range(n.value)]
