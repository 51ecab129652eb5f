"""Generates the golden fixtures from the reference's own shipped outputs.

Run once in a checkout that has the reference tree (it is not needed at test
time):  python tests/golden/make_golden.py /path/to/tracer_code

Inputs (files of the reference repository):
  Trestart               unformatted record xg(-3:203), zg(-3:203),
                         T(-2:202,-2:202), SF(-2:202,-2:202) written by
                         print_restart (main.f90:301-320) at the end of the
                         shipped 200x200 run
  stats.dat              one row per step (basics.f90:283-314); its last row
                         is computed from the same T and SF (main.f90:181-190)
  viscosity_smoother.dat n_eta, eig_fine, n_temp of that step
                         (basics.f90:316-322)
  main.f90               the shipped inputs (parsed for the values the pin
                         needs, so none are typed in by hand)
  equalize.dat           '(g20.8,15(i10))' rows (composition.f90:568-574),
                         kept verbatim with stats.dat's and
                         viscosity_smoother.dat's rows for the text formatters
Outputs: tests/golden/trestart_200.npz and tests/golden/golden.json (which
also records the Trestart file's size and sha256, the byte-exact pin of the
restart writer).
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_trestart(path: str, nx: int = 200, nz: int = 200, span: int = 2, span_interp: int = 1):
    b = open(path, "rb").read()
    n0 = struct.unpack("<i", b[:4])[0]
    n1 = struct.unpack("<i", b[-4:])[0]
    assert n0 == n1 == len(b) - 8, "single unformatted record expected"
    a = np.frombuffer(b[4:-4], dtype="<f8")
    ng_x = nx + 1 + 2 * (span + span_interp)
    ng_z = nz + 1 + 2 * (span + span_interp)
    xg, zg = a[:ng_x], a[ng_x:ng_x + ng_z]
    off = ng_x + ng_z
    nT = (nx + 1 + 2 * span) * (nz + 1 + 2 * span)
    T = a[off:off + nT].reshape(nz + 1 + 2 * span, nx + 1 + 2 * span)
    SF = a[off + nT:off + 2 * nT].reshape(nz + 1 + 2 * span, nx + 1 + 2 * span)
    assert off + 2 * nT == a.size
    return xg.copy(), zg.copy(), T.copy(), SF.copy()


def parse_inputs(main_f90: str) -> dict:
    want = ["RaT", "aspect", "nx", "nz", "order", "tolerance", "Nmulti", "grids", "eig_ratio", "vis_iter", "torder",
            "courant", "courantT", "courant_stream", "comp", "tracer", "ivis", "visP", "visT", "delta_visT",
            "yield", "yield_gradient", "yield_depth", "eig_ratio_min", "non_Newtonian", "iterate_order", "mingrid",
            "Tbot", "Vbc"]
    vals = {}
    for line in open(main_f90):
        s = line.split("!!")[0].strip()
        m = re.match(r"^([A-Za-z_]+)\s*=\s*(.+)$", s)
        if not m or m.group(1) not in want or m.group(1) in vals:
            continue
        expr = m.group(2).replace("d", "e").replace("D", "e")
        vals[m.group(1)] = float(eval(expr, {"__builtins__": {}}, {}))
    return vals


def main(ref: str) -> None:
    xg, zg, T, SF = read_trestart(os.path.join(ref, "Trestart"))
    stats_rows = [l.split() for l in open(os.path.join(ref, "stats.dat")) if l.strip()]
    vis_rows = [l.split() for l in open(os.path.join(ref, "viscosity_smoother.dat")) if l.strip()]
    last = stats_rows[-1]
    cols = ["time", "Tavg", "vrms", "Nu", "Nu_bot", "RaT_avg", "mobility", "strain_max", "q1", "q2", "q3", "q4"]
    stats_last = {c: float(last[i]) for i, c in enumerate(cols)}
    stats_last.update(empty_cells=int(last[12]), tracer_min=int(last[13]), tracer_max=int(last[14]))
    vl = vis_rows[-1]
    vis_last = {"time": float(vl[0]), "n_eta": int(vl[1]), "eig_fine": float(vl[2]), "n_temp": int(vl[3])}
    dt_rows = [float(r[0]) for r in stats_rows]
    golden = {
        "source": "reference repository files Trestart, stats.dat, viscosity_smoother.dat, main.f90",
        "inputs": parse_inputs(os.path.join(ref, "main.f90")),
        "stats_last": stats_last,
        "viscosity_smoother_last": vis_last,
        "stats_dt": dt_rows[1] - dt_rows[0],
        "stats_rows": len(stats_rows),
        "print_digits": 8,
        "trestart_bytes": os.path.getsize(os.path.join(ref, "Trestart")),
        "trestart_sha256": hashlib.sha256(open(os.path.join(ref, "Trestart"), "rb").read()).hexdigest(),
        # the shipped text rows verbatim (pins of the gfortran-style formatters)
        "text_lines": {f: [l for l in open(os.path.join(ref, f)).read().split("\n") if l.strip()]
                       for f in ("stats.dat", "viscosity_smoother.dat", "equalize.dat")},
    }
    np.savez_compressed(os.path.join(HERE, "trestart_200.npz"), xg=xg, zg=zg, T=T, SF=SF)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "trestart_200.npz"), "and golden.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/tracer_code")
    main(sys.argv[1])
