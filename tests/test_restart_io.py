"""Restart files in the reference's format (tc_restart_* of tracer_gpu.h;
print_restart main.f90:301-330, build_grid grid.f90:55-108).  Host-only
calls through the C ABI: no GPU needed.

  - the writer reproduces the reference's shipped Trestart (200x200,
    RaT /= 0, comp = 0: xg, zg, T, SF) byte for byte, with the coordinates
    from tc_restart_grid;
  - the reader returns the shipped arrays and refuses files that do not
    hold exactly the expected record;
  - the comp = 1 layouts (Cnew between T and SF, type fastest; no T when
    RaT = 0; restart_tracers = rtr, str, Ttype) and the temperature-tracer
    layouts (rtr, str[, Ttype], Ttr) round trip and have the byte layout of
    one gfortran unformatted record.
"""
import hashlib
import os
import struct

import numpy as np
import pytest

from tracer_code_gb300 import build as tcbuild
from tracer_code_gb300.abi import TracerError

ARG, TOO_LARGE = 1, 12


@pytest.fixture(scope="module")
def rs():
    tcbuild.build()
    from tracer_code_gb300 import restart
    return restart


def record(path):
    b = open(path, "rb").read()
    n0 = struct.unpack("<i", b[:4])[0]
    n1 = struct.unpack("<i", b[-4:])[0]
    assert n0 == n1 == len(b) - 8
    return b[4:-4]


def test_grid_equals_shipped_coordinates(rs, golden):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "trestart_200.npz"))
    xg, zg = rs.grid(200, 200, golden["inputs"]["aspect"])
    assert np.array_equal(xg, z["xg"]) and np.array_equal(zg, z["zg"])


def test_writer_reproduces_shipped_trestart(rs, golden, tmp_path):
    xg, zg = rs.grid(200, 200, golden["inputs"]["aspect"])
    p = tmp_path / "Trestart"
    rs.write_trestart(p, xg, zg, golden["SF"], T=golden["T"])
    b = open(p, "rb").read()
    assert len(b) == golden["trestart_bytes"]
    assert hashlib.sha256(b).hexdigest() == golden["trestart_sha256"]


def test_reader_returns_shipped_arrays(rs, golden, tmp_path):
    xg, zg = rs.grid(200, 200, golden["inputs"]["aspect"])
    p = tmp_path / "Trestart"
    rs.write_trestart(p, xg, zg, golden["SF"], T=golden["T"])
    d = rs.read_trestart(p, 200, 200, ntype=0, thermal=True)
    assert np.array_equal(d["T"], golden["T"]) and np.array_equal(d["SF"], golden["SF"])
    assert np.array_equal(d["xg"], xg) and np.array_equal(d["zg"], zg)
    # the same file read as another grid, another type count or without T
    for kw in ({"nx": 199, "nz": 200}, {"nx": 200, "nz": 201}):
        with pytest.raises(TracerError) as e:
            rs.read_trestart(p, kw["nx"], kw["nz"], ntype=0, thermal=True)
        assert e.value.status == ARG
    with pytest.raises(TracerError):
        rs.read_trestart(p, 200, 200, ntype=1, thermal=True)
    with pytest.raises(TracerError):
        rs.read_trestart(p, 200, 200, ntype=0, thermal=False)


@pytest.mark.parametrize("thermal,ntype", [(True, 1), (True, 3), (False, 2)])
def test_comp_layout_round_trip(rs, tmp_path, thermal, ntype):
    nx, nz = 24, 10
    rng = np.random.default_rng(ntype)
    shp = (nz + 5, nx + 5)
    xg, zg = rs.grid(nx, nz, 2.4)
    T = rng.random(shp) if thermal else None
    Cn = rng.random(shp + (ntype,))
    SF = rng.standard_normal(shp)
    p = tmp_path / "Trestart"
    rs.write_trestart(p, xg, zg, SF, T=T, Cnew=Cn)
    payload = np.frombuffer(record(p), "<f8")
    parts = [xg, zg] + ([T.ravel()] if thermal else []) + [Cn.ravel(), SF.ravel()]
    assert np.array_equal(payload, np.concatenate(parts))
    d = rs.read_trestart(p, nx, nz, ntype=ntype, thermal=thermal)
    assert np.array_equal(d["Cnew"], Cn) and np.array_equal(d["SF"], SF)
    if thermal:
        assert np.array_equal(d["T"], T)


def test_tracer_file_round_trip(rs, tmp_path):
    rng = np.random.default_rng(3)
    n = 1001
    r, s = rng.random(n) * 2.4, rng.random(n)
    t = rng.integers(0, 3, n).astype(np.int32)
    p = tmp_path / "restart_tracers"
    rs.write_tracers(p, r, s, t)
    b = record(p)
    assert len(b) == 20 * n
    assert np.array_equal(np.frombuffer(b[:8 * n], "<f8"), r)
    assert np.array_equal(np.frombuffer(b[8 * n:16 * n], "<f8"), s)
    assert np.array_equal(np.frombuffer(b[16 * n:], "<i4"), t)
    d = rs.read_tracers(p, n)
    assert np.array_equal(d["rtr"], r) and np.array_equal(d["str"], s) and np.array_equal(d["Ttype"], t)
    with pytest.raises(TracerError):
        rs.read_tracers(p, n + 1)
    # temperature tracers: rtr, str, Ttr (comp = 0) and rtr, str, Ttype, Ttr (comp = 1)
    Tt = rng.random(n)
    for with_type in (False, True):
        rs.write_tracers(p, r, s, t if with_type else None, Tt)
        b = record(p)
        assert len(b) == (28 if with_type else 24) * n
        assert np.array_equal(np.frombuffer(b[-8 * n:], "<f8"), Tt)
        d = rs.read_tracers(p, n, Ttype=with_type, Ttr=True)
        assert np.array_equal(d["Ttr"], Tt) and np.array_equal(d["rtr"], r)
        if with_type:
            assert np.array_equal(d["Ttype"], t)
        with pytest.raises(TracerError):
            rs.read_tracers(p, n, Ttype=not with_type, Ttr=True)


def test_damaged_files_are_refused(rs, tmp_path):
    nx, nz = 8, 4
    shp = (nz + 5, nx + 5)
    xg, zg = rs.grid(nx, nz, 1.0)
    p = tmp_path / "Trestart"
    rs.write_trestart(p, xg, zg, np.zeros(shp), T=np.ones(shp))
    good = open(p, "rb").read()
    bad = {
        "truncated": good[:-12],
        "trailer": good[:-4] + struct.pack("<i", len(good) - 7),
        "header": struct.pack("<i", len(good)) + good[4:],
        "two records": good + good,
        "empty": b"",
    }
    for name, b in bad.items():
        q = tmp_path / name.replace(" ", "_")
        q.write_bytes(b)
        with pytest.raises(TracerError) as e:
            rs.read_trestart(q, nx, nz, ntype=0, thermal=True)
        assert e.value.status == ARG, name
    with pytest.raises(TracerError):
        rs.read_trestart(tmp_path / "missing", nx, nz)


def test_argument_checks(rs, tmp_path):
    from tracer_code_gb300 import load_library
    L = load_library()
    xg, zg = rs.grid(8, 4, 1.0)
    sf = np.zeros((9, 13))
    ptr = rs._p
    q = os.fsencode(tmp_path / "x")
    assert L.tc_restart_write(q, 8, 4, 5, 1, ptr(xg), ptr(zg), ptr(sf), ptr(sf), ptr(sf)) == ARG  # ntype > 4
    assert L.tc_restart_write(q, 8, 4, 1, 1, ptr(xg), ptr(zg), ptr(sf), None, ptr(sf)) == ARG  # Cnew missing
    assert L.tc_restart_write(q, 8, 4, 0, 1, ptr(xg), ptr(zg), None, None, ptr(sf)) == ARG  # T missing
    assert L.tc_restart_write(q, 0, 4, 0, 0, ptr(xg), ptr(zg), None, None, ptr(sf)) == ARG
    assert L.tc_restart_tracers_write(q, 0, ptr(xg), ptr(xg), ptr(xg), None) == ARG
    assert L.tc_restart_tracers_write(q, 4, ptr(xg), ptr(xg), None, None) == ARG  # neither Ttype nor Ttr
    # a record of 2^31 bytes or more is refused before any array is touched
    big = 1 << 28
    assert L.tc_restart_tracers_write(q, big, ptr(xg), ptr(xg), ptr(xg), None) == TOO_LARGE
    assert not os.path.exists(tmp_path / "x")
