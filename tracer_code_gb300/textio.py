"""The reference's text outputs through the C ABI (tc_format_* and
tc_write_snapshot in include/tracer_gpu.h): stats.dat and
viscosity_smoother.dat rows (basics.f90:283-322) and the T1xxxx snapshot
(main.f90:237-270), written as gfortran's formatted WRITE lays them out.
The formatters are host-only calls, usable without a GPU."""
from __future__ import annotations

import ctypes as C

from .abi import StatsRow, TracerError


def _lib():
    from . import load_library
    return load_library()


def format_g(x: float, w: int, d: int, e: int = 0) -> str:
    """One real under Gw.d (e = 0) or Gw.dEe."""
    buf = C.create_string_buffer(w + 1)
    n = _lib().tc_format_g(float(x), w, d, e, buf)
    if n < 0:
        raise TracerError(1, "format_g", f"G{w}.{d}E{e} out of range")
    return buf.raw[:n].decode()


def _row(row) -> StatsRow:
    if isinstance(row, StatsRow):
        return row
    r = StatsRow()
    for name, _ in StatsRow._fields_:
        if name in row:
            v = row[name]
            if hasattr(v, "__len__"):
                arr = getattr(r, name)
                for i, x in enumerate(v):
                    arr[i] = x
            else:
                setattr(r, name, v)
    return r


def stats_line(row, comp: int, tracer: int, ntype: int, RaT: float) -> str:
    """The stats.dat row (basics.f90:283-314, local_time = 0), without newline."""
    buf = C.create_string_buffer(1024)
    r = _row(row)
    st = _lib().tc_format_stats_line(C.byref(r), comp, tracer, ntype, float(RaT), buf, len(buf))
    if st:
        raise TracerError(st, "format_stats_line")
    return buf.value.decode()


def vis_line(row, comp: int, ntype: int, RaT: float) -> str:
    """The viscosity_smoother.dat row (basics.f90:316-322), without newline."""
    buf = C.create_string_buffer(256)
    r = _row(row)
    st = _lib().tc_format_vis_line(C.byref(r), comp, ntype, float(RaT), buf, len(buf))
    if st:
        raise TracerError(st, "format_vis_line")
    return buf.value.decode()


def equalize_line(time: float, row) -> str:
    """The equalize.dat row (composition.f90:568-574) of a tc_equalize_row result."""
    arr = (C.c_int64 * len(row))(*[int(v) for v in row])
    buf = C.create_string_buffer(512)
    st = _lib().tc_format_equalize_line(float(time), arr, len(row), buf, len(buf))
    if st:
        raise TracerError(st, "format_equalize_line")
    return buf.value.decode()
