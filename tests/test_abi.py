"""The C-ABI library loads on a machine without a GPU and exports every
function include/*.h declares (tracer_gpu.h: the solver, tracer_nn.h: the
learned guess); ctypes structs match the C layout.  No compute call is made
here."""
import ctypes as C
import os
import re

import pytest

from tracer_code_gb300 import build as tcbuild
from tracer_code_gb300.abi import Info, Params, StatsRow, default_params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    tcbuild.build()
    import tracer_code_gb300 as tc
    return tc.load_library()


def header_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        txt = re.sub(r"/\*.*?\*/", "", open(os.path.join(inc, f)).read(), flags=re.S)
        names |= set(re.findall(r"\b((?:tc|tcnn)_[a-z_0-9]+)\s*\(", txt))
    return sorted(names)


def test_header_declares_the_drop_in_entry_points():
    names = header_functions()
    for n in ["tc_create", "tc_destroy", "tc_upload_state", "tc_download_state", "tc_multigrid",
              "tc_compute_velocities", "tc_stats", "tc_energy_time", "tc_step"]:
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_sizes_match(lib):
    sizes = (C.c_int32 * 3)()
    lib.tc_abi_sizes(sizes)
    assert tuple(sizes) == (C.sizeof(Params), C.sizeof(StatsRow), C.sizeof(Info))


def test_default_params_agree(lib):
    a = Params()
    lib.tc_default_params(C.byref(a))
    b = default_params()
    for name, _ in Params._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if hasattr(va, "__len__"):
            va, vb = list(va), list(vb)
        assert va == vb, name
