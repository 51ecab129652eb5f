"""Ensemble of independent cases stepped together (tc_ensemble_run,
tc_ensemble_step).

Each case is its own handle on its own CUDA stream.  With graph=True (the
default) one ensemble step is one CUDA graph launch: every case's captured
timestep is a branch of one graph, so the GPU executes the cases side by
side (the small cases' latency-bound smoother launches fill SMs the large
cases leave idle) with one host synchronisation per step; the first step,
and any step a case is not ready to capture, runs tc_step on every case
from a pool of host threads instead.  Each case may carry the learned
initial guess (its own network instance, since a network holds one image's
activations); with a network the cases use the learned start and the
network's direction in their correction.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import Simulation, TracerError, load_library, state
from .abi import STATUS, StatsRow, config_1024x256


def case_params(i: int, seed: int = 1):
    """Case i of the 64-case mix: grids 256x64 / 512x128 / 1024x256 in turn,
    10..25 tracers per cell, Ra log-uniform in 1e5..1e7, B uniform in
    0.2..1.0, viscosity contrast log-uniform in 1e2..1e5, mixed precision,
    coarse corrections from zero, the bottom-of-cycle matrix and the windowed
    correction; drawn from a generator seeded by (seed, i)."""
    rng = np.random.default_rng([seed, i])
    sizes = [(256, 64, 4), (512, 128, 5), (1024, 256, 6)]
    nx, nz, grids = sizes[i % 3]
    p = config_1024x256()
    p.nx, p.nz, p.grids = nx, nz, grids
    p.tpc = 10 + (i * 7) % 16
    ra = 10.0 ** rng.uniform(5.0, 7.0)
    p.RaT = ra
    p.RaC[0] = rng.uniform(0.2, 1.0) * ra
    p.visT = 10.0 ** rng.uniform(2.0, 5.0)
    p.mg_zero_coarse = 1
    p.mg_coarse_matrix = 1
    p.solver_precision = 1
    p.cycle_correction = 3
    return p


class Ensemble:
    def __init__(self, params: list, seeds: list | None = None, weights: str | None = None,
                 autotune: bool = True, graph: bool = True, nthreads: int | None = None):
        from . import learned
        self.L = load_library()
        self.graph = None
        if graph:
            e = C.c_void_p()
            r = self.L.tc_ensemble_create(nthreads or len(params), C.byref(e))
            if r != 0:
                raise TracerError(r, "tc_ensemble_create")
            self.graph = e
        self.sims = []
        self.nets = []
        self.params = params
        for i, p in enumerate(params):
            q = p.copy()
            if weights is not None:
                # the learned start and the network's direction in the correction
                q.learned_guess = 3
                if q.cycle_correction in (1, 3):
                    q.cycle_correction += 1
            sim = Simulation(q)
            if weights is not None:
                net = learned.Net(1, q.nz, q.nx)
                net.load(weights)
                learned.attach(sim, net)
                self.nets.append(net)
            sim.upload(state.initial_state(q, seed=(seeds[i] if seeds else 1 + i)))
            self.sims.append(sim)
        self.tuning = None
        if autotune:
            # launch shapes depend on the level sizes and the precision only:
            # tune the first case of each kind, apply its shapes to the rest
            tuned = {}
            self.tuning = []
            for s, p in zip(self.sims, params):
                key = (p.nx, p.nz, s.info.grids, p.solver_precision, p.Nmulti)
                if key in tuned:
                    s.set_launch_shapes(tuned[key])
                else:
                    tuned[key] = s.autotune()
                self.tuning.append(tuned[key])
        self.n = len(self.sims)
        self.ntr = [s.ntr for s in self.sims]
        # cases still running; a case stops (as the reference's run stops) at
        # its first error status, which is kept in self.stopped
        self.active = list(range(self.n))
        self.stopped = {}

    def step(self, nthreads: int | None = None, strict: bool = True):
        """One tc_step on every active case.  strict: raise on any error;
        otherwise cases that fail are stopped and left out of later steps.
        Returns per-case (rows, cycles, dts), None for cases not stepped."""
        idx = list(self.active)
        n = len(idx)
        rows_o, cyc_o, dt_o = [None] * self.n, [None] * self.n, [None] * self.n
        if n == 0:
            return rows_o, cyc_o, dt_o
        hs = (C.c_void_p * n)(*[self.sims[i].h.value for i in idx])
        rows = (StatsRow * n)()
        cyc = (C.c_int32 * n)()
        dts = (C.c_double * n)()
        st = (C.c_int32 * n)()
        if self.graph is not None:
            r = self.L.tc_ensemble_run(self.graph, hs, n, C.cast(rows, C.c_void_p), C.cast(cyc, C.c_void_p),
                                       C.cast(dts, C.c_void_p), C.cast(st, C.c_void_p))
        else:
            r = self.L.tc_ensemble_step(hs, n, nthreads or n, C.cast(rows, C.c_void_p), C.cast(cyc, C.c_void_p),
                                        C.cast(dts, C.c_void_p), C.cast(st, C.c_void_p))
        if r != 0 and strict:
            bad = [(idx[j], STATUS.get(st[j], st[j])) for j in range(n) if st[j] != 0]
            raise TracerError(r, f"tc_ensemble_step: {bad}")
        for j, i in enumerate(idx):
            if st[j] != 0:
                self.stopped[i] = STATUS.get(st[j], st[j])
                self.active.remove(i)
                continue
            rows_o[i], cyc_o[i], dt_o[i] = rows[j].as_dict(), cyc[j], dts[j]
        return rows_o, cyc_o, dt_o

    def graph_info(self):
        """(steps run as one graph launch, steps run by the thread pool)."""
        if self.graph is None:
            return 0, 0
        g = C.c_int64(0); e = C.c_int64(0)
        self.L.tc_ensemble_info(self.graph, C.byref(g), C.byref(e))
        return g.value, e.value

    def close(self):
        if self.graph is not None:
            self.L.tc_ensemble_destroy(self.graph)
            self.graph = None
        for s in self.sims:
            s.close()
        for nt in self.nets:
            nt.close()
        self.sims, self.nets = [], []
