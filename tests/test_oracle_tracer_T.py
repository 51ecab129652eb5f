"""Temperature tracers (tracer = 1) in the CPU restatement: the per-volume
mean Tratio of tracers_to_corners (composition.f90:669-790).

The per-volume sums are exact (each Ttr as a 128-bit fixed-point integer at
2^-64, rounded to double once), so:
  - Tratio equals the correctly rounded exact mean (computed here with
    Python fractions) in every interior volume that holds tracers, and T
    (the upload's empty-volume fallback) in the others;
  - Tratio does not change when the tracers are stored in another order;
  - equal temperatures give that temperature back exactly.
"""
from fractions import Fraction

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from tests.cases import case_1024_like, fresh_state

SP = 2


def _case(comp, nx=32, nz=8, tpc=3):
    p = case_1024_like(nx=nx, nz=nz, grids=2, tpc=tpc)
    p.tracer, p.comp, p.mg_zero_coarse = 1, comp, 1
    return p


def _exact_means(p, st):
    dr, ds = p.aspect / p.nx, 1.0 / p.nz
    sums, cnt = {}, {}
    for r, s, t in zip(st["rtr"], st["str"], st["Ttr"]):
        key = (int(np.floor(r / dr + 0.5)), int(np.floor(s / ds + 0.5)))
        sums[key] = sums.get(key, Fraction(0)) + Fraction(float(t))
        cnt[key] = cnt.get(key, 0) + 1
    return {k: float(v) / cnt[k] for k, v in sums.items()}


@pytest.mark.parametrize("comp", [0, 1])
def test_tratio_is_the_exact_mean(comp):
    p = _case(comp)
    st = fresh_state(p, seed=6)
    rng = np.random.default_rng(1)
    # temperatures with full 53-bit mantissas and both signs, all >= 2^-11 in magnitude
    st["Ttr"] = rng.uniform(0.001, 1.5, st["rtr"].size) * rng.choice([-1.0, 1.0], st["rtr"].size)
    o = Oracle(p)
    o.upload(st)
    Tr = o.get("Tratio")
    T = o.get("T")
    means = _exact_means(p, st)
    checked = 0
    for i in range(p.nx + 1):
        for k in range(1, p.nz):  # rows 0 and nz take the wall values of enforceBCs
            v = Tr[k + SP, i + SP]
            if (i, k) in means:
                assert v == means[(i, k)], (i, k)
                checked += 1
            else:
                assert v == T[k + SP, i + SP]
    assert checked > 0.9 * (p.nx + 1) * (p.nz - 1)


def test_tratio_does_not_depend_on_tracer_order():
    p = _case(1)
    st = fresh_state(p, seed=8)
    rng = np.random.default_rng(2)
    st["Ttr"] = rng.random(st["rtr"].size)
    perm = rng.permutation(st["rtr"].size)
    st2 = dict(st)
    for k in ("rtr", "str", "Ttype", "Ttr"):
        st2[k] = np.ascontiguousarray(st[k][perm])
    a, b = Oracle(p), Oracle(p)
    a.upload(st)
    b.upload(st2)
    assert np.array_equal(a.get("Tratio"), b.get("Tratio"))
    assert np.array_equal(a.counts(), b.counts())


def test_equal_temperatures_come_back_exactly():
    p = _case(0)
    st = fresh_state(p, seed=9)
    st["Ttr"] = np.full(st["rtr"].size, 0.3)
    o = Oracle(p)
    o.upload(st)
    Tr = o.get("Tratio")
    ne = o.counts().sum(axis=2)
    inner = (ne[SP + 1:SP + p.nz, SP:SP + p.nx + 1] > 0)
    assert np.all(Tr[SP + 1:SP + p.nz, SP:SP + p.nx + 1][inner] == 0.3)


def test_steps_run_and_keep_the_tracer_state():
    """A few steps with temperature tracers: positions stay inside, Ttr stays
    bounded by the initial range plus conduction overshoot, the grid T is
    Tratio after each step, and the counts cover every tracer."""
    p = case_1024_like(nx=128, nz=32, grids=4, tpc=4)
    p.tracer, p.comp, p.mg_zero_coarse = 1, 0, 1
    o = Oracle(p)
    o.upload(fresh_state(p, seed=3))
    for _ in range(2):
        row, q, dt = o.step()
        assert q > 0 and dt > 0
        d = o.download()
        assert np.array_equal(d["T"], o.get("Tratio"))
        assert d["Ttr"].min() > -0.1 and d["Ttr"].max() < 1.1
        assert int(o.counts()[SP:SP + p.nz + 1, SP:SP + p.nx + 1].sum()) == o.ntr
        assert row["tracer_min"] >= 0 and row["tracer_max"] > 0
