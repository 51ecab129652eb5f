"""The reference's restart files through the C ABI (tc_restart_* in
include/tracer_gpu.h): host-only calls, usable without a GPU.

Arrays follow the library's layouts: fields (nz+5, nx+5) with i fastest,
Cnew (nz+5, nx+5, ntype) with the type fastest, coordinates xg(-3:nx+3) and
zg(-3:nz+3).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .abi import TracerError

SPAN, SPAN_X = 2, 3


def _lib():
    from . import load_library
    return load_library()


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def grid(nx: int, nz: int, aspect: float):
    """build_grid's uniform xg, zg with ghost mirrors (grid.f90:46-54, 97-108)."""
    xg = np.empty(nx + 1 + 2 * SPAN_X)
    zg = np.empty(nz + 1 + 2 * SPAN_X)
    _lib().tc_restart_grid(nx, nz, float(aspect), _p(xg), _p(zg))
    return xg, zg


def write_trestart(path, xg, zg, SF, T=None, Cnew=None) -> None:
    """print_restart's Trestart record (main.f90:305-320)."""
    nx = len(xg) - 1 - 2 * SPAN_X
    nz = len(zg) - 1 - 2 * SPAN_X
    shp = (nz + 1 + 2 * SPAN, nx + 1 + 2 * SPAN)
    arrs = [np.ascontiguousarray(a, np.float64) if a is not None else None for a in (xg, zg, T, Cnew, SF)]
    xg, zg, T, Cnew, SF = arrs
    if SF.shape != shp or (T is not None and T.shape != shp) or (Cnew is not None and Cnew.shape[:2] != shp):
        raise TracerError(1, "write_trestart", f"fields must have shape {shp}")
    ntype = 0 if Cnew is None else (Cnew.shape[2] if Cnew.ndim == 3 else 1)
    st = _lib().tc_restart_write(os.fsencode(path), nx, nz, ntype, int(T is not None), _p(xg), _p(zg), _p(T),
                                 _p(Cnew), _p(SF))
    if st:
        raise TracerError(st, "write_trestart")


def read_trestart(path, nx: int, nz: int, ntype: int = 0, thermal: bool = True) -> dict:
    """build_grid's Trestart read (grid.f90:55-66) for the given grid."""
    shp = (nz + 1 + 2 * SPAN, nx + 1 + 2 * SPAN)
    xg = np.empty(nx + 1 + 2 * SPAN_X); zg = np.empty(nz + 1 + 2 * SPAN_X)
    SF = np.empty(shp)
    T = np.empty(shp) if thermal else None
    Cn = np.empty(shp + (ntype,)) if ntype else None
    st = _lib().tc_restart_read(os.fsencode(path), nx, nz, ntype, int(thermal), _p(xg), _p(zg), _p(T), _p(Cn),
                                _p(SF))
    if st:
        raise TracerError(st, "read_trestart")
    out = {"xg": xg, "zg": zg, "SF": SF}
    if thermal:
        out["T"] = T
    if ntype:
        out["Cnew"] = Cn
    return out


def write_tracers(path, rtr, str_, Ttype=None, Ttr=None) -> None:
    """print_restart's restart_tracers record (main.f90:321-330): rtr, str,
    then Ttype (comp = 1) and/or Ttr (tracer = 1)."""
    r = np.ascontiguousarray(rtr, np.float64)
    s = np.ascontiguousarray(str_, np.float64)
    t = None if Ttype is None else np.ascontiguousarray(Ttype, np.int32)
    tt = None if Ttr is None else np.ascontiguousarray(Ttr, np.float64)
    if r.size != s.size or (t is not None and t.size != r.size) or (tt is not None and tt.size != r.size):
        raise TracerError(1, "write_tracers", "rtr, str, Ttype, Ttr must have one length")
    st = _lib().tc_restart_tracers_write(os.fsencode(path), r.size, _p(r), _p(s), _p(t), _p(tt))
    if st:
        raise TracerError(st, "write_tracers")


def read_tracers(path, ntr: int, Ttype: bool = True, Ttr: bool = False) -> dict:
    """build_grid's restart_tracers read (grid.f90:74-84) for the given record layout."""
    r = np.empty(ntr); s = np.empty(ntr)
    t = np.empty(ntr, np.int32) if Ttype else None
    tt = np.empty(ntr) if Ttr else None
    st = _lib().tc_restart_tracers_read(os.fsencode(path), ntr, _p(r), _p(s), _p(t), _p(tt))
    if st:
        raise TracerError(st, "read_tracers")
    out = {"rtr": r, "str": s}
    if Ttype:
        out["Ttype"] = t
    if Ttr:
        out["Ttr"] = tt
    return out
