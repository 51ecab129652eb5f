"""Oracle trajectories for the GPU parity tests (run once on a CPU; the
fixtures are committed, the oracle is not needed at test time):

  traj_128x128.json    the 128x128 plain case (aspect 1, Ra 1e5, B 0.5,
                       isoviscous, dense layer z < 0.2, 20 tracers per cell,
                       multigrid to 1e-8): 100 steps
  traj_1024x256.json   the 1024x256 case (aspect 4, Ra 1e7, B 0.8,
                       eta = exp(-ln(1e4) T) x 10 in enriched material,
                       25 tracers per cell, 6 levels, coarse corrections
                       restarting from zero): 20 steps; its per-volume
                       counts after the last step go to
                       traj_1024x256_counts.npz

Each file holds, per step, the stats.dat row (Nu, Vrms, Tavg, Nu_bot,
Cavg, empty_cells, tracer_min, tracer_max), the W-cycles of the step and dt,
with the seeded initial state's seed, a checksum of the per-volume tracer
counts after every step, and after the last step the counts' sum and
checksum.

    python tests/golden/make_trajectories.py [128|1024]
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import Oracle  # noqa: E402
from tracer_code_gb300 import config_1024x256, config_plain_128, state  # noqa: E402

KEYS = ("Nu", "vrms", "Tavg", "Nu_bot", "empty_cells", "tracer_min", "tracer_max")


def case(name: str):
    if name == "128":
        return config_plain_128(), 100, "traj_128x128.json"
    p = config_1024x256()
    p.mg_zero_coarse = 1
    return p, 20, "traj_1024x256.json"


def checksum(counts: np.ndarray) -> int:
    c = counts.astype(np.int64).ravel()
    return int((c * (np.arange(c.size) % 9973 + 1)).sum())


def run(name: str, seed: int = 1) -> None:
    p, steps, fname = case(name)
    o = Oracle(p)
    o.upload(state.initial_state(p, seed=seed))
    rows = []
    t0 = time.time()
    for n in range(steps):
        row, q, dt = o.step()
        r = {k: row[k] for k in KEYS}
        r["Cavg"] = row["Cavg"][0]
        r.update(cycles=int(q), dt=float(dt), counts_checksum=checksum(o.counts()))
        rows.append(r)
        print(name, n, q, row["Nu"], row["vrms"], round(time.time() - t0, 1), flush=True)
    counts = o.counts()
    out = {"case": name, "nx": p.nx, "nz": p.nz, "tpc": p.tpc, "seed": seed, "steps": steps, "rows": rows,
           "counts_sum": int(counts.sum()),
           "counts_checksum": checksum(counts)}
    with open(os.path.join(HERE, fname), "w") as f:
        json.dump(out, f, indent=1)
    if name != "128":
        np.savez_compressed(os.path.join(HERE, fname.replace(".json", "_counts.npz")), counts=counts.astype(np.int16))
    print("wrote", fname)


if __name__ == "__main__":
    for name in (sys.argv[1:] or ["128", "1024"]):
        run(name)
