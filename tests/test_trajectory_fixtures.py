"""The committed oracle trajectories (tests/golden/traj_*.json, made by
tests/golden/make_trajectories.py) are the oracle's own output: its first
steps recomputed here give the same rows."""
import json
import os

import pytest

from oracle.pyoracle import Oracle
from tracer_code_gb300 import config_plain_128, state

HERE = os.path.join(os.path.dirname(__file__), "golden")


def test_128x128_trajectory_prefix_is_the_oracle():
    with open(os.path.join(HERE, "traj_128x128.json")) as f:
        d = json.load(f)
    assert d["steps"] == len(d["rows"]) == 100
    p = config_plain_128()
    o = Oracle(p)
    o.upload(state.initial_state(p, seed=d["seed"]))
    for n in range(2):
        row, q, dt = o.step()
        ref = d["rows"][n]
        assert q == ref["cycles"] and dt == pytest.approx(ref["dt"], rel=1e-12)
        for k in ("Nu", "vrms", "Tavg", "Nu_bot"):
            assert row[k] == pytest.approx(ref[k], rel=1e-12), k
        assert row["Cavg"][0] == pytest.approx(ref["Cavg"], rel=1e-12)


def test_1024x256_trajectory_is_complete():
    import numpy as np
    with open(os.path.join(HERE, "traj_1024x256.json")) as f:
        d = json.load(f)
    assert d["steps"] == len(d["rows"]) == 20 and d["nx"] == 1024 and d["nz"] == 256
    assert d["counts_sum"] >= (d["nx"] + 1) * (d["nz"] + 1) * d["tpc"]  # interior plus mirrored ghosts
    # the final per-volume counts file matches the recorded sum and checksum
    counts = np.load(os.path.join(HERE, "traj_1024x256_counts.npz"))["counts"].astype(np.int64)
    assert int(counts.sum()) == d["counts_sum"]
    c = counts.ravel()
    assert int((c * (np.arange(c.size) % 9973 + 1)).sum()) == d["counts_checksum"]
    assert d["rows"][-1]["counts_checksum"] == d["counts_checksum"]
