"""Benchmark: timesteps/s of the per-timestep hot path at 1024x256 cells with
25 tracers per cell (6,585,625 tracers), multigrid to 1e-8 relative residual.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one pass of the reference main loop body (main.f90:181-204):
multigrid, compute_velocities, stats, energy_time (RK4: three more multigrid
solves, four tracer RK stages, four tracer-ratio composition passes).

ours: W untimed steps, then K steps timed with CUDA events on the library's
stream (barrier + synchronize on both sides, max over ranks).  N>1 runs N
independent replicas (one case per GPU; the path does not shard).  Inputs
are larger than L2 (the tracer state alone is 6.6M x 8 FP64 arrays).
Prints one JSON line (rank 0) with the contract keys plus roofline,
cpu_baseline, e2e, clocks and gpu_launches.

reference: the CPU restatement of the reference (oracle/, OpenMP on all host
cores) on the same workload.  Its timed steps are whole timesteps from the
seeded initial state (every multigrid solve to the 1e-8 test, cycles
counted, four RK stages, four tracer-ratio passes), measured with a wall
clock.  A whole CPU timestep takes about a minute, so the arm times as many
of the K requested steps as fit REF_BUDGET_S (at least one) and reports the
number it timed in "steps" (the request in "steps_requested"); its W warm-up
steps are bounded (one W-cycle each on a separate copy of the state).

Other modes, each printing its own JSON line: --ensemble N (N independent
cases of three grid sizes stepped together, one CUDA graph launch per
ensemble step), --config3 N (the 2048x512 case, mixed precision against
FP64 over N steps), and the --profile-* cases that end by themselves under
ncu.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "timesteps/s 1024x256 grid, 6.5M tracers: learned+mixed vs plain MG @ 1e-8 resid"
UNIT = "timesteps/s"
# wall-clock budget of the reference arm's timed whole CPU timesteps (s): it
# stops after the step that crosses it (so at least one step is timed)
REF_BUDGET_S = 150.0
# W-cycle caps of the two CPU multigrid calls of one bounded sample (their
# difference gives the time per cycle, about 10 s of CPU work per sample)
CPU_SAMPLE_CYCLES = (2, 24)
# dram__bytes_read.sum + dram__bytes_write.sum per launch of the level-1
# smoother kernels from one ncu capture each (cold cache; the FP64 kernel in
# profiles/multigrid_solve_1024x256.md, the FP32 field sweep k_sweep_g32 in
# profiles/k_sweep_g32_1024x256.md).
SWEEP_DRAM_BYTES = 34.0e6
SWEEP32_DRAM_BYTES = 8.65e6


def workload_params(solver: str = "plain"):
    from tracer_code_gb300 import config_1024x256
    p = config_1024x256()
    p.mg_zero_coarse = 1
    p.mg_coarse_matrix = 1
    p.solver_precision = 1 if solver == "mixed" else 0
    return p


SOLVER_DESC = {
    "plain": "plain FP64 multigrid (W-cycle, Chebyshev-Richardson smoother, banded LU coarse solve), "
             "coarse corrections restart from zero (mg_zero_coarse=1); the bottom of each W-cycle (level-5 "
             "visits and coarsest solves) applied as its precomputed exact linear map (mg_coarse_matrix=1)",
    "mixed": "mixed-precision multigrid: the same W-cycle with FP32 smoother, residuals and transfers on levels "
             "1..grids-1 inside FP64 defect correction (FP64 level-1 residual, streamfunction and updates, FP64 "
             "coarse solve), same 1e-8 test",
    "learned": "learned + mixed: the mixed-precision multigrid with the encoder-decoder (BF16 tcgen05 network "
               "trained at 512x128) supplying its predicted change of each solve as (a) the start, scaled to the "
               "residual-minimising multiple (learned_guess=3), and (b) a direction of the correction after every "
               "level-1 visit, whose other directions are psi's changes over the last four W-cycles (a windowed "
               "Krylov acceleration of the W-cycle), with coefficients minimising the L1-weighted residual "
               "(cycle_correction=4); same 1e-8 test",
    "corr": "mixed + windowed correction without the network: the same correction after every level-1 visit "
            "over psi's changes of the last four W-cycles only (cycle_correction=3); same 1e-8 test",
    "corr1": "mixed + one-direction correction: the correction after every level-1 visit along psi's change "
             "over the last W-cycle only (cycle_correction=1); same 1e-8 test",
}
GUESS_WEIGHTS = os.path.join(ROOT, "tracer_code_gb300", "weights", "guess_512x128.npy")


def workload_desc(p, solver: str) -> dict:
    ntr = (p.nx + 1) * (p.nz + 1) * p.tpc
    return {
        "workload": f"{p.nx}x{p.nz} cells, aspect {p.aspect:g}, {p.tpc} tracers/cell ({ntr:,} tracers), "
                    f"Ra={p.RaT:g}, B={p.RaC[0] / p.RaT:g}, dense layer z<{p.dlayer:g}, "
                    f"eta=exp(-ln({p.visT:g})T)*10 in enriched, RK4, multigrid {p.grids} levels to {p.tolerance:g}",
        "grid": f"{p.nx}x{p.nz}",
        "tracers": ntr,
        "solver": SOLVER_DESC[solver],
        "l2": "inputs larger than L2 (tracer state 6.6M x 8 FP64 arrays = 421 MB)",
        "parallelism": "replicas (one independent case per GPU)",
    }


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        out_dir = os.environ.get("TC_CLOCK_LOG_DIR", "/tmp")
        self.path = os.path.join(out_dir, f"tc_clocks_{os.getpid()}_{index}.csv")

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        try:
            rows = [l.strip().split(",") for l in open(self.path) if l.strip()]
        except Exception:
            rows = []
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() in ("active", "1"):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_sample(p, threads: int, cycles_per_step: float, seed: int = 1) -> dict:
    """Bounded sample of the CPU restatement on the full workload; returns the
    assembled timestep time and its parts."""
    from oracle.pyoracle import Oracle
    from tracer_code_gb300 import TracerError, state
    st = state.initial_state(p, seed=seed)
    q = p.copy()
    times = {}
    lo, hi = CPU_SAMPLE_CYCLES
    for cap in (lo, hi):
        q.max_cycles = cap
        o2 = Oracle(q, threads=threads)
        o2.upload(st)
        t0 = time.perf_counter()
        try:
            o2.multigrid()
        except TracerError as e:
            if e.status != 3:
                raise
        times[cap] = time.perf_counter() - t0
        if cap == hi:
            o2.compute_velocities()
            qq = q.copy()
            qq.RK_update = 0
            o3 = Oracle(qq, threads=threads)
            o3.upload(st)
            o3.set("SF", o2.download()["SF"])
            o3.compute_velocities()
            t0 = time.perf_counter()
            o3.energy_time()
            times["rk_step_no_resolve"] = time.perf_counter() - t0
            r = o3.download()
            t0 = time.perf_counter()
            o3.tracers_to_corners(r["rtr"], r["str"])
            times["tracers_to_corners"] = time.perf_counter() - t0
            o3.close()
        o2.close()
    per_cycle = max((times[hi] - times[lo]) / (hi - lo), 1e-9)
    fixed = max(times[lo] - lo * per_cycle, 0.0)
    step = 4 * fixed + cycles_per_step * per_cycle + times["rk_step_no_resolve"] + 3 * times["tracers_to_corners"]
    return {"step_s": step, "per_cycle_s": per_cycle, "per_solve_fixed_s": fixed,
            "rk_step_no_resolve_s": times["rk_step_no_resolve"], "tracers_to_corners_s": times["tracers_to_corners"],
            "sample_s": sum(v for v in times.values())}


def run_reference(args, rank: int, world: int):
    """The reference arm: whole CPU timesteps of the restatement on all host
    cores, timed with a wall clock (rank 0 only; other ranks do no work)."""
    if rank != 0:
        return
    from oracle.pyoracle import Oracle
    from tracer_code_gb300 import TracerError, state
    p = workload_params()
    threads = os.cpu_count() or 1
    st = state.initial_state(p, seed=1)
    # bounded warm-up steps (thread pool, first touch): one W-cycle each on a copy
    q = p.copy()
    q.max_cycles = 1
    ow = Oracle(q, threads=threads)
    ow.upload(st)
    for _ in range(args.warmup):
        try:
            ow.multigrid()
        except TracerError as e:
            if e.status != 3:
                raise
    ow.close()
    o = Oracle(p, threads=threads)
    o.upload(st)
    times, cycles = [], []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, qc, _ = o.step()
        times.append(time.perf_counter() - t0)
        cycles.append(int(qc))
        if time.perf_counter() - t_all >= REF_BUDGET_S:
            break
    o.close()
    total = sum(times)
    value = len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": len(times),
        "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(workload_desc(p, "plain"), mg_zero_coarse=p.mg_zero_coarse,
                       solver="the reference's plain FP64 multigrid restated on the CPU (W-cycle, Chebyshev-"
                              "Richardson smoother, banded LU coarse solve, every level visit and coarse solve "
                              "carried out), coarse corrections restart from zero (mg_zero_coarse=1)"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{len(times)} whole timesteps of the CPU restatement from the seeded initial "
                                   f"state (every solve to the 1e-8 test), wall clock; W-cycles per step {cycles}; "
                                   f"steps timed = those of the {args.steps} requested that fit {REF_BUDGET_S:g} s",
                         "step_s": times, "cycles_per_step": cycles},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def timed_steps(sim, stream, steps: int, warmup: int, barrier):
    """W untimed steps, then K steps between CUDA events on the library's
    stream; returns (ms, cycles of the timed steps, cycles of the warm-up,
    kernel launches in the timed region)."""
    import torch
    from tracer_code_gb300 import Simulation
    warm = [sim.step()[1] for _ in range(warmup)]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    n0 = Simulation.kernel_launches()
    e0.record(stream)
    cyc = [sim.step()[1] for _ in range(steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    return e0.elapsed_time(e1), cyc, warm, Simulation.kernel_launches() - n0


# the reference's 6-level W-cycle (multigrid_cycle.f90:91-92), steps p = 1..42
W_TABLE6 = [1, 2, 3, 4, 5, 6, 5, 6, 5, 4, 5, 6, 5, 4, 3, 4, 5, 6, 5, 4, 3, 2, 3, 4, 5, 6, 5, 4, 3, 4, 5, 6, 5, 4,
            5, 6, 5, 6, 5, 4, 3, 2]


def visits_per_cycle(grids: int) -> dict:
    if grids != 6:
        raise ValueError("the bench workload runs 6 levels")
    return {l: W_TABLE6.count(l) for l in range(1, grids + 1)}


def bottom_patterns(grids: int) -> dict:
    """Descents into level grids-1 per W-cycle, keyed by the coarsest solves
    each makes before the cycle leaves level grids-1 again."""
    t = W_TABLE6 if grids == 6 else None
    if t is None:
        raise ValueError("the bench workload runs 6 levels")
    S, out = grids - 1, {}
    n = len(t)
    for i in range(n):
        if t[i] == S and t[i - 1] == S - 1:
            k, j = 0, i
            while t[(j + 1) % n] >= S:
                j += 1
                k += t[j % n] == grids
            out[k] = out.get(k, 0) + 1
    return out


def level_points(p, level: int) -> int:
    f = 2 ** (level - 1)
    return (p.nx // f - 1) * (p.nz // f - 1)


def cycle_profile(sim, p, fp32: bool) -> dict:
    """Per-level share of one W-cycle, timed live on the library's stream:
    each level's whole smoother visit (tc_time_visit: its kernels, replayed
    back to back) times its visits per cycle; the level whose visits take
    the largest share holds the dominant kernel.  Algorithmic bytes of a
    visit = Nmulti sweeps x (88 B FP64 | 44 B FP32) x interior points."""
    from tracer_code_gb300 import Simulation
    visits = visits_per_cycle(p.grids)
    bsweep = 44.0 if fp32 else 88.0
    rows = []
    matrix = bool(getattr(p, "mg_coarse_matrix", 0))
    top = p.grids - 1 if matrix else p.grids
    for lvl in range(1, top):
        reps = 3 if lvl == 1 else 20
        n0 = Simulation.kernel_launches()
        ms = sim.time_visit(lvl, reps)
        launches = (Simulation.kernel_launches() - n0) / (reps + 1)
        pts = level_points(p, lvl)
        rows.append({"level": lvl, "points": pts, "visits_per_cycle": visits[lvl], "ms_per_visit": ms,
                     "launches_per_visit": launches, "ms_per_cycle": ms * visits[lvl],
                     "alg_bytes_per_visit": p.Nmulti * bsweep * pts})
    bottom = None
    if matrix:
        # level grids-1 and the coarsest solves: one product per descent
        S = p.grids - 1
        pat = bottom_patterns(p.grids)
        nS = level_points(p, S)
        ms = {k: sim.time_subcycle(k, 50) for k in pat}
        es = 4.0 if fp32 else 8.0
        bottom = {"level": S, "points": nS, "products_per_cycle": pat,
                  "ms_per_product": ms, "ms_per_cycle": sum(pat[k] * ms[k] for k in pat),
                  "alg_bytes_per_product": es * nS * nS + 2 * es * nS,
                  "replaces": f"{visits[S]} visits of level {S} and {visits[p.grids]} coarsest solves per cycle"}
        rows.append({"level": S, "points": nS, "visits_per_cycle": sum(pat.values()),
                     "ms_per_visit": bottom["ms_per_cycle"] / sum(pat.values()), "launches_per_visit": 1.0,
                     "ms_per_cycle": bottom["ms_per_cycle"],
                     "alg_bytes_per_visit": bottom["alg_bytes_per_product"], "matrix": True})
    tot = sum(r["ms_per_cycle"] for r in rows)
    for r in rows:
        r["share_of_smoothing"] = r["ms_per_cycle"] / tot
    return {"levels": rows, "coarse_solves_per_cycle": 0 if matrix else visits[p.grids], "bottom_matrix": bottom}


def dominant_roofline(sim, p, prof: dict, fp32: bool) -> dict:
    """Roofline of the kernel that takes the largest share of a W-cycle: at
    level 1 the per-sweep smoother launch (70 per visit), below it the
    level's visit (one cluster launch per visit where it fuses)."""
    peak, src = peaks()
    dom = max(prof["levels"], key=lambda r: r["ms_per_cycle"])
    lvl, pts = dom["level"], dom["points"]
    if lvl == 1:
        return sweep_roofline(sim, p, fp32) | {"share_of_smoothing": dom["share_of_smoothing"]}
    per_launch_ms = dom["ms_per_visit"] / max(dom["launches_per_visit"], 1.0)
    alg = dom["alg_bytes_per_visit"] / max(dom["launches_per_visit"], 1.0)
    achieved = alg / (per_launch_ms * 1e-3) / 1e9
    if dom.get("matrix"):
        return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None, "kernel": f"k_subcycle_apply (level {lvl}, {pts}x{pts} matrix)",
                "alg_bytes_per_launch": alg, "kernel_ms": per_launch_ms,
                "share_of_smoothing": dom["share_of_smoothing"],
                "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs burst)" if src == "measured" else "fallback"}
    fused = abs(dom["launches_per_visit"] - 1.0) < 1e-9
    kname = ("k_visit_cluster" if fused else "smoother launches") + f"<{'float' if fp32 else 'double'}>"
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None,
            "kernel": f"{kname} (level {lvl}, {pts} points, {p.Nmulti} sweeps per launch)" if fused else
                      f"{kname} (level {lvl}, {pts} points)",
            "alg_bytes_per_launch": alg, "kernel_ms": per_launch_ms,
            "share_of_smoothing": dom["share_of_smoothing"],
            "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs burst)" if src == "measured" else "fallback 6.8 TB/s",
            "note": "latency bound: the level lives in the shared memory and registers of one thread-block "
                    "cluster for the whole visit, so each sweep costs one compute-exchange-wait chain; "
                    "achieved = the sweeps' algorithmic bytes over the launch time (traffic null: the level "
                    "is read from HBM once per visit)"}


def step_roofline(p, prof: dict, cycles_per_step: float, ms_per_step: float, fp32: bool) -> dict:
    """Whole-timestep algorithmic bytes (model of the per-unit figures above)
    over the measured step time: smoother sweeps, residuals (72 B/pt), the
    FP64 level-1 bridges of the mixed solve, the correction after each
    level-1 visit, tracer RK stages (64 B/tracer) and tracer-ratio passes
    (20 B/tracer + 20 B/volume)."""
    peak, _ = peaks()
    bsweep = 44.0 if fp32 else 88.0
    per_cycle = 0.0
    for r in prof["levels"]:
        if r.get("matrix"):
            per_cycle += r["visits_per_cycle"] * r["alg_bytes_per_visit"]
        else:
            per_cycle += r["visits_per_cycle"] * (p.Nmulti * bsweep + (36.0 if fp32 else 72.0)) * r["points"]
    if fp32:
        per_cycle += (72.0 + 24.0 + 72.0) * level_points(p, 1)  # residual_to32, update64, FP64 residual
    cc = int(getattr(p, "cycle_correction", 0))
    if cc >= 3:
        # windowed correction: 13 FP64 coefficients, psi, prev, RHS, three
        # stored images and the network direction read, the new change and
        # its image written; then four changes, the direction and psi read,
        # psi and prev written
        per_cycle += (104.0 + 24.0 + 24.0 + 16.0 + 48.0 + 16.0) * level_points(p, 1)
    elif cc >= 1:
        per_cycle += (104.0 + 32.0 + 40.0) * level_points(p, 1)
    ntr = (p.nx + 1) * (p.nz + 1) * p.tpc
    vols = (p.nx + 1) * (p.nz + 1)
    tracer = 4 * 64.0 * ntr + 4 * (20.0 * ntr + 20.0 * vols)
    total = cycles_per_step * per_cycle + tracer
    achieved = total / (ms_per_step * 1e-3) / 1e9
    return {"alg_bytes_per_step": total, "multigrid_bytes_per_cycle": per_cycle, "tracer_bytes_per_step": tracer,
            "cycles_per_step": cycles_per_step, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak}


def sweep_roofline(sim, p, fp32: bool) -> dict:
    """Level-1 smoother sweep timed live on the library's stream."""
    sweep_ms = sim.time_sweep(1, 70)
    ni, nk = p.nx - 1, p.nz - 1
    alg_bytes = (44.0 if fp32 else 88.0) * ni * nk
    achieved = alg_bytes / (sweep_ms * 1e-3) / 1e9
    peak, src = peaks()
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": SWEEP32_DRAM_BYTES if fp32 else SWEEP_DRAM_BYTES,
            "kernel": ("k_sweep_g32" if fp32 else "k_sweep") + f" (level 1, {ni}x{nk} points)",
            "alg_bytes_per_launch": alg_bytes, "kernel_ms": sweep_ms,
            "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs burst)" if src == "measured" else "fallback 6.8 TB/s",
            "note": ("FP32: 44 B/pt algorithmic (the FP64 88 B/pt count at half width); the field sweep reads five "
                     "viscosity fields, dt, RHS and psi (a cold launch reads 8.65 MB = 33 B/pt from DRAM) and forms "
                     "the 13 coefficients in registers; between sweeps the level-1 FP32 working set is L2-resident"
                     if fp32 else
                     "FP64-pipe bound on GB300: 15 FP64 ops/point/sweep at 1.2 TFLOP/s")}


def shipped_params():
    """The reference's own shipped main.f90 inputs (parsed from it into
    tests/golden/golden.json): 200x200, aspect 1, 2 levels, tolerance 1e-3,
    plastic viscosity (ivis 3) with the non-Newtonian iteration, temperature
    tracers (30 per volume), tracer repositioning; TRA reproduces a
    16-thread OpenMP run."""
    from tracer_code_gb300 import default_params
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        inp = json.load(f)["inputs"]
    p = default_params()
    p.nx, p.nz, p.aspect, p.order = int(inp["nx"]), int(inp["nz"]), inp["aspect"], int(inp["order"])
    p.comp, p.ntype, p.tracer, p.tpc = int(inp["comp"]), 0, int(inp["tracer"]), 30
    p.equalize, p.equalize_threads = 1, 16
    p.ivis, p.non_Newtonian = int(inp["ivis"]), int(inp["non_Newtonian"])
    p.visT, p.visP, p.delta_visT = inp["visT"], inp["visP"], inp["delta_visT"]
    p.yield_, p.yield_gradient, p.yield_depth = inp["yield"], inp["yield_gradient"], inp["yield_depth"]
    p.RaT, p.tolerance, p.grids, p.Nmulti = inp["RaT"], inp["tolerance"], int(inp["grids"]), int(inp["Nmulti"])
    p.eig_ratio, p.eig_ratio_min, p.vis_iter = inp["eig_ratio"], inp["eig_ratio_min"], int(inp["vis_iter"])
    p.torder, p.courant, p.courantT = int(inp["torder"]), inp["courant"], inp["courantT"]
    p.courant_stream, p.iterate_order, p.mingrid = inp["courant_stream"], int(inp["iterate_order"]), int(inp["mingrid"])
    p.Tbot, p.Vbc = int(inp["Tbot"]), int(inp["Vbc"])
    return p


def shipped_config_rates(stream, steps: int, warmup: int, cpu: bool) -> dict:
    """Timesteps/s of the reference's shipped configuration on this GPU (and,
    for one step, the CPU restatement on the host cores) from a seeded state."""
    import torch
    from tracer_code_gb300 import Simulation, state
    p = shipped_params()
    st = state.initial_state(p, seed=1)
    sim = Simulation(p, stream=stream.cuda_stream)
    sim.upload(st)
    for _ in range(warmup):
        sim.step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rows = [sim.step() for _ in range(steps)]
    torch.cuda.synchronize()
    gpu_s = (time.perf_counter() - t0) / steps
    out = {"config": "reference main.f90 inputs: 200x200, comp=0, tracer=1 (30/volume), equalize=1 (16 threads), "
                     "ivis=3, non_Newtonian=1, 2 levels, tolerance 1e-3; seeded synthetic state",
           "gpu_timesteps_per_s": 1.0 / gpu_s, "cycles_per_step": [r[1] for r in rows],
           "tracers_moved_last_step": (sim.equalize_row() or [0, 0, 0, 0, 0])[4]}
    sim.close()
    if cpu:
        from oracle.pyoracle import Oracle
        o = Oracle(p, threads=os.cpu_count() or 1)
        o.upload(st)
        o.step()
        t0 = time.perf_counter()
        o.step()
        out["cpu_restatement_timesteps_per_s"] = 1.0 / (time.perf_counter() - t0)
        out["cpu_cores"] = os.cpu_count() or 1
        out["cpu_sample"] = "second step from the same state (the first moves no tracers)"
        o.close()
    return out


def replica_rate(units_per_rank: float, seconds_local: float, world: int, max_over_ranks) -> float:
    """Whole-job throughput of N independent replicas: the units all ranks
    processed over the slowest rank's time (each rank runs the same work, so
    the units are world * units_per_rank).  max_over_ranks reduces a float
    over the process group (identity for one rank)."""
    return world * units_per_rank / max_over_ranks(seconds_local)


def run_ours(args, rank: int, world: int, local_rank: int):
    import numpy as np
    import torch
    import torch.distributed as dist
    from tracer_code_gb300 import Simulation, state

    torch.cuda.set_device(local_rank)
    stream = torch.cuda.Stream()

    def barrier():
        if world > 1:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        if world > 1:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    from tracer_code_gb300 import learned
    # headline arm: mixed-precision solver with the learned start and the
    # learned coarse-level correction
    p = workload_params("mixed")
    p.learned_guess = 3
    p.cycle_correction = 4
    st = state.initial_state(p, seed=1 + rank)
    sim = Simulation(p, stream=stream.cuda_stream)
    net = learned.Net(1, p.nz, p.nx, stream=stream.cuda_stream)
    net.load(GUESS_WEIGHTS)
    learned.attach(sim, net)
    sim.upload(st)
    shapes = sim.autotune()  # launch shapes per level, timed on this GPU (tc_autotune)
    sim.set_step_graph(args.step_graph)
    with ClockSampler(local_rank) as clk:
        ms, solves, cycles, launches = timed_steps(sim, stream, args.steps, args.warmup, barrier)
    guess_used, guess_offered = learned.guess_stats(sim)
    # the same handle with every timestep as one graph launch (the other mode)
    sim.set_step_graph(not args.step_graph)
    g0 = sim.step_graph_info()[0]
    # untimed steps up to and including the next tracer sort, so that both of
    # the step's graphs (with and without the sort) are captured untimed
    t = args.warmup + args.steps
    ival = max(int(p.tracer_sort_interval), 1)
    w_other = max(2, (ival - t % ival) % ival + 1)
    msg, solvesg, _, _ = timed_steps(sim, stream, args.steps, w_other, barrier)
    other_mode = {"timesteps_per_s": replica_rate(args.steps, msg * 1e-3, world, max_over_ranks),
                  "ms_per_step": msg / args.steps, "cycles_per_step": solvesg,
                  "steps_as_one_graph_launch": sim.step_graph_info()[0] - g0}
    sim.set_step_graph(args.step_graph)
    ms_max = max_over_ranks(ms)
    value = replica_rate(args.steps, ms * 1e-3, world, max_over_ranks)
    prof = cycle_profile(sim, p, fp32=True)
    roof = dominant_roofline(sim, p, prof, fp32=True)
    roof_l1 = sweep_roofline(sim, p, fp32=True)
    step_roof = step_roofline(p, prof, statistics.mean(solves), ms_max / args.steps, fp32=True)
    # end to end: the same steps through tc_step_host with pinned host state
    host = {}
    dl = sim.download()
    for key in ("T", "SF", "Cnew", "rtr", "str", "Ttype"):
        a = dl[key]
        pt = torch.empty(a.shape, dtype=torch.float64 if a.dtype == np.float64 else torch.int32).pin_memory()
        host[key] = pt.numpy()
        host[key][...] = a
    h2d = sum(host[k].nbytes for k in ("T", "SF", "Cnew", "rtr", "str", "Ttype"))
    d2h = sum(host[k].nbytes for k in ("T", "SF", "Cnew", "rtr", "str"))
    k_e2e = args.steps
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(k_e2e):
        sim.step_host(host)
    torch.cuda.synchronize()
    e2e_value = replica_rate(k_e2e, time.perf_counter() - t0, world, max_over_ranks)
    sim.close()
    net.close()
    # ablations: the same windowed correction without the network's
    # direction, and the one-direction correction
    pc = workload_params("mixed")
    pc.cycle_correction = 3
    simc = Simulation(pc, stream=stream.cuda_stream)
    simc.upload(st)
    simc.autotune()
    simc.set_step_graph(args.step_graph)
    msc, solvesc, _, _ = timed_steps(simc, stream, args.steps, args.warmup, barrier)
    corr_value = replica_rate(args.steps, msc * 1e-3, world, max_over_ranks)
    simc.close()
    pc1 = workload_params("mixed")
    pc1.cycle_correction = 1
    simc1 = Simulation(pc1, stream=stream.cuda_stream)
    simc1.upload(st)
    simc1.autotune()
    simc1.set_step_graph(args.step_graph)
    msc1, solvesc1, _, _ = timed_steps(simc1, stream, args.steps, args.warmup, barrier)
    corr1_value = replica_rate(args.steps, msc1 * 1e-3, world, max_over_ranks)
    simc1.close()
    # the same mixed solver without the network and without the correction
    pm = workload_params("mixed")
    simm = Simulation(pm, stream=stream.cuda_stream)
    simm.upload(st)
    simm.autotune()
    simm.set_step_graph(args.step_graph)
    msm, solvesm, _, _ = timed_steps(simm, stream, args.steps, args.warmup, barrier)
    mixed_value = replica_rate(args.steps, msm * 1e-3, world, max_over_ranks)
    simm.close()
    # comparison arm: plain FP64 multigrid on the same initial state
    pp = workload_params("plain")
    sim0 = Simulation(pp, stream=stream.cuda_stream)
    sim0.upload(st)
    sim0.autotune()
    sim0.set_step_graph(args.step_graph)
    ms0, solves0, cycles0, _ = timed_steps(sim0, stream, args.steps, args.warmup, barrier)
    plain_value = replica_rate(args.steps, ms0 * 1e-3, world, max_over_ranks)
    prof0 = cycle_profile(sim0, pp, fp32=False)
    roof0 = dominant_roofline(sim0, pp, prof0, fp32=False)
    roof0_l1 = sweep_roofline(sim0, pp, fp32=False)
    step_roof0 = step_roofline(pp, prof0, statistics.mean(solves0), ms0 / args.steps, fp32=False)
    sim0.close()
    shipped = shipped_config_rates(stream, 3, 1, cpu=(rank == 0 and not args.no_cpu_baseline)) if rank == 0 else None
    if rank == 0:
        cfg = dict(workload_desc(p, "learned"), mg_zero_coarse=p.mg_zero_coarse,
                   mg_zero_coarse_note="coarse-level corrections restart from zero when a level receives a new "
                                       "restricted residual (the reference keeps them; with 6 levels its W-cycle "
                                       "stalls on this workload); both arms and the CPU reference arm use it",
                   launch_shapes={"tuned_by": "tc_autotune on this GPU, every arm",
                                  "per_level_block_x_block_y_visit": shapes},
                   step_graph={"timed_arms_as_one_graph_launch_per_step": bool(args.step_graph),
                               ("eager_steps" if args.step_graph else "graph_steps"): dict(
                                   other_mode, note="the headline arm's handle, continued for another "
                                                    f"{args.steps} timed steps after {w_other} untimed ones"),
                               "note": "a graph step (tc_set_step_graph) is the whole timestep as one CUDA graph "
                                       "launch, its convergence and filter loops conditional WHILE nodes and "
                                       "the host's reads of the step's scalars made once after it; its results "
                                       "equal the eager step's bit for bit.  The eager step (default) reads "
                                       "the scalars once per solve, filter call and stop test"},
                   cycles_per_step=solves, warmup_cycles_per_step=cycles,
                   w_cycle_profile=prof, level1_sweep_roofline=roof_l1, step_roofline=step_roof,
                   tracer_rk_stages_per_s=value * 4 * ((p.nx + 1) * (p.nz + 1) * p.tpc),
                   learned_guess={"weights": os.path.relpath(GUESS_WEIGHTS, ROOT), "solves_offered": guess_offered,
                                  "solves_started_from_guess": guess_used},
                   cycle_correction_without_network={"timesteps_per_s": corr_value, "ms_per_step": msc / args.steps,
                                                     "cycles_per_step": solvesc, "solver": SOLVER_DESC["corr"]},
                   one_direction_correction={"timesteps_per_s": corr1_value, "ms_per_step": msc1 / args.steps,
                                             "cycles_per_step": solvesc1, "solver": SOLVER_DESC["corr1"]},
                   mixed_without_guess={"timesteps_per_s": mixed_value, "ms_per_step": msm / args.steps,
                                        "cycles_per_step": solvesm,
                                        "solver": "the mixed-precision multigrid alone (no network, no correction)"},
                   learned_gain={"cycles_vs_mixed_alone": sum(solves) / max(sum(solvesm), 1),
                                 "cycles_vs_correction_without_network": sum(solves) / max(sum(solvesc), 1)},
                   plain_fp64={"timesteps_per_s": plain_value, "ms_per_step": ms0 / args.steps,
                               "cycles_per_step": solves0, "solver": SOLVER_DESC["plain"], "roofline": roof0,
                               "level1_sweep_roofline": roof0_l1, "step_roofline": step_roof0,
                               "w_cycle_profile": prof0},
                   speedup_vs_plain_fp64=value / plain_value,
                   reference_shipped_config=shipped)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded conductive T + uniform tracers)",
            "config": cfg,
            "roofline": roof,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "steps": k_e2e, "api": "tc_step_host (C ABI, pinned host arrays)"},
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
        }
        if not args.no_cpu_baseline:
            cps = float(statistics.mean(solves0))
            r = cpu_sample(pp, os.cpu_count() or 1, cps)
            line["cpu_baseline"] = {"value": 1.0 / r["step_s"], "unit": UNIT, "cores": os.cpu_count() or 1,
                                    "kind": "port",
                                    "sample": f"CPU restatement (FP64), full workload: multigrid capped at {CPU_SAMPLE_CYCLES[0]} and {CPU_SAMPLE_CYCLES[1]} "
                                              f"W-cycles, one RK4 step without re-solves, one tracer-ratio pass "
                                              f"({r['sample_s']:.1f} s); timestep = 4*fixed + {cps:g} cycles + RK "
                                              f"+ 3 ratio passes",
                                    "parts": r}
        print(json.dumps(line), flush=True)


def run_ensemble(args):
    """Batched ensemble: args.ensemble cases (tracer_code_gb300.ensemble.case_params), mixed solver with
    the bottom-of-cycle matrix, the learned start and the windowed correction with the network's
    direction, autotuned launch shapes per case, stepped together by one graph launch per step
    (tc_ensemble_run)."""
    import torch
    from tracer_code_gb300.ensemble import Ensemble, case_params
    t0 = time.time()
    params = [case_params(i) for i in range(args.ensemble)]
    ens = Ensemble(params, weights=GUESS_WEIGHTS, autotune=True, graph=not args.no_step_graph)
    setup_s = time.time() - t0
    # cases whose run stops (tracers leaving the domain, a diverging solve:
    # the reference's `stop` sites) stop during the warm-up and are left out
    for _ in range(args.warmup):
        ens.step(strict=False)
    # a case that stopped in the last warm-up step changes the case list, so
    # the next step captures a new ensemble graph: take that step untimed too
    extra_warmup = 0
    while extra_warmup < 5:
        before = list(ens.active)
        ens.step(strict=False)
        extra_warmup += 1
        if ens.active == before:
            break
    torch.cuda.synchronize()
    active = list(ens.active)
    t1 = time.perf_counter()
    cyc = []
    for _ in range(args.steps):
        _, c, _ = ens.step(strict=False)
        cyc.append([c[i] for i in active])
    torch.cuda.synchronize()
    el = time.perf_counter() - t1
    if ens.active != active:
        raise RuntimeError(f"cases stopped inside the timed steps: {sorted(set(active) - set(ens.active))}")
    graph_steps, pool_steps = ens.graph_info()
    ntr = sum(ens.ntr[i] for i in active)
    sizes = {}
    for p in params:
        k = f"{p.nx}x{p.nz}"
        sizes[k] = sizes.get(k, 0) + 1
    line = {
        "metric": "tracer*RK-stages/s, batched ensemble", "value": ntr * 4 * args.steps / el,
        "unit": "tracer*RK-stages/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic (seeded per case)",
        "config": {"workload": f"{args.ensemble} independent cases, grids {sizes}, 10-25 tracers/cell, "
                               f"Ra 1e5-1e7, B 0.2-1.0, viscosity contrast 1e2-1e5",
                   "solver": "mixed precision, bottom-of-cycle matrix, learned start (learned_guess=3) and "
                             "windowed correction with the network's direction (cycle_correction=4)",
                   "tracers_total": ntr, "cases_timed": len(active),
                   "cases_stopped_in_warmup": {str(k): v for k, v in sorted(ens.stopped.items())},
                   "per_case_timesteps_per_s": args.steps / el,
                   "cycles_per_step_per_case": cyc, "setup_s": setup_s,
                   "execution": ("one CUDA graph launch per ensemble timestep (tc_ensemble_run): every case's "
                                 "captured step, with its convergence and filter loops as conditional WHILE "
                                 "nodes, is a branch of one graph forked onto the cases' streams; the first "
                                 "step, and steps after a case stops, run tc_step per case from a host thread "
                                 "pool; launch shapes from tc_autotune")
                                if not args.no_step_graph else
                                "one handle and stream per case, tc_step issued by a host thread pool "
                                "(tc_ensemble_step); launch shapes from tc_autotune",
                   "steps_as_one_graph_launch": graph_steps, "steps_by_thread_pool": pool_steps,
                   "extra_warmup_steps": extra_warmup},
    }
    ens.close()
    print(json.dumps(line), flush=True)


def config3_params(prec: int):
    """The 2048x512 case (aspect 4, 40 tracers per cell, Ra 1e8, B 1.0,
    contrast 1e6 x 30) with coarse corrections from zero, the bottom-of-cycle
    matrix and the windowed correction (without it the W-cycle stops with an
    abnormally high residual on this case, in the oracle as here)."""
    from tracer_code_gb300.abi import config_2048x512
    p = config_2048x512()
    p.mg_zero_coarse = 1
    p.mg_coarse_matrix = 1
    p.cycle_correction = 3
    p.solver_precision = prec
    return p


def run_config3(args):
    """Mixed precision against FP64 on the 2048x512 case: both solvers step the
    same seeded state args.config3 timesteps (every solve to the same 1e-8
    test); prints per-arm timesteps/s and W-cycles per step and the mixed
    solver's error against the FP64 one in SF, Nu, Vrms and the tracer mass
    (the mean C) at every 10th step and at the end."""
    import numpy as np
    from tracer_code_gb300 import Simulation, state
    n = args.config3
    st = state.initial_state(config3_params(1), seed=1)
    arms = {}
    for name, prec in (("fp64", 0), ("mixed", 1)):
        sim = Simulation(config3_params(prec))
        sim.upload(st)
        rows, cyc = [], []
        t0 = time.perf_counter()
        for _ in range(n):
            row, q, _ = sim.step()
            rows.append(row)
            cyc.append(q)
        el = time.perf_counter() - t0
        d = sim.download()
        arms[name] = {"rows": rows, "cycles": cyc, "s": el, "SF": d["SF"], "T": d["T"]}
        sim.close()
    a, b = arms["mixed"], arms["fp64"]

    def rel(x, y):
        return abs(x - y) / abs(y) if y != 0 else abs(x - y)

    checks = []
    for k in list(range(9, n, 10)) + ([n - 1] if (n - 1) % 10 != 9 else []):
        ra, rb = a["rows"][k], b["rows"][k]
        checks.append({"step": k + 1, "Nu": rel(ra["Nu"], rb["Nu"]), "vrms": rel(ra["vrms"], rb["vrms"]),
                       "mass": rel(ra["Cavg"][0], rb["Cavg"][0])})
    sf_err = float(np.abs(a["SF"] - b["SF"]).max() / np.abs(b["SF"]).max())
    t_err = float(np.abs(a["T"] - b["T"]).max())
    line = {
        "metric": "2048x512 mixed-precision error against FP64 and timesteps/s", "n_gpus": 1, "steps": n,
        "data": "synthetic (seeded conductive T + uniform tracers)",
        "config": {"workload": "2048x512 cells, aspect 4, 40 tracers/cell (42,045,480 tracers), Ra=1e8, B=1.0, "
                               "eta=exp(-ln(1e6)T)*30 in enriched, RK4, multigrid 6 levels to 1e-8",
                   "solver": "mg_zero_coarse=1, bottom-of-cycle matrix, windowed correction (cycle_correction=3); "
                             "mixed = FP32 smoother in FP64 defect correction"},
        "fp64": {"timesteps_per_s": n / b["s"], "cycles_per_step": b["cycles"]},
        "mixed": {"timesteps_per_s": n / a["s"], "cycles_per_step": a["cycles"]},
        "mixed_vs_fp64": {"SF_max_rel_at_end": sf_err, "T_max_abs_at_end": t_err,
                          "max_rel": {k: max(c[k] for c in checks) for k in ("Nu", "vrms", "mass")},
                          "at_steps": checks},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--step-graph", action="store_true",
                    help="time the single-case arms with every timestep as one CUDA graph launch")
    ap.add_argument("--no-step-graph", action="store_true",
                    help="ensemble: step the cases from a host thread pool instead of one graph launch per step")
    ap.add_argument("--profile-step", metavar="NXxNZ", default=None,
                    help="one timestep of the workload's physics on a smaller grid (for ncu), e.g. 512x128")
    ap.add_argument("--profile-shipped", action="store_true",
                    help="two timesteps of the reference's shipped configuration (for ncu)")
    ap.add_argument("--profile-solve", action="store_true",
                    help="profiling case: upload the workload, run one multigrid solve, exit")
    ap.add_argument("--solver", default="plain", choices=["plain", "mixed", "learned"],
                    help="solver of --profile-solve / --profile-step (learned: the headline arm's, with the "
                         "committed network)")
    ap.add_argument("--profile-net", action="store_true",
                    help="profiling case: one guess-network forward and backward on one 1024x256 image, exit")
    ap.add_argument("--ensemble", type=int, default=0, metavar="N",
                    help="instead of the headline: N independent cases (256x64/512x128/1024x256 in turn, "
                         "randomised physics) stepped together; prints aggregate tracer*RK-stages/s")
    ap.add_argument("--config3", type=int, default=0, metavar="N",
                    help="instead of the headline: the 2048x512 case, mixed precision against FP64 over N steps")
    args = ap.parse_args()
    if args.config3:
        run_config3(args)
        return
    if args.ensemble:
        run_ensemble(args)
        return
    if args.profile_net:
        import numpy as np
        import torch
        from tracer_code_gb300 import learned
        p = workload_params("mixed")
        net = learned.Net(1, p.nz, p.nx)
        net.load(GUESS_WEIGHTS)
        rng = np.random.default_rng(1)
        raw = torch.from_numpy(rng.normal(size=(1, 3, p.nz, p.nx)).astype(np.float32)).cuda()
        sf = torch.from_numpy(rng.normal(size=(1, p.nz, p.nx)).astype(np.float32)).cuda()
        out = torch.empty((1, p.nz, p.nx), dtype=torch.float32, device="cuda")
        net.forward(raw.data_ptr(), 1, out.data_ptr())
        loss = net.loss_backward(raw.data_ptr(), sf.data_ptr(), 1)
        torch.cuda.synchronize()
        print(json.dumps({"profile_net": True, "loss": loss}), flush=True)
        net.close()
        return
    if args.profile_step:
        from tracer_code_gb300 import Simulation, state, scaled_config
        nx, nz = (int(v) for v in args.profile_step.lower().split("x"))
        p = scaled_config(workload_params("mixed" if args.solver == "learned" else args.solver), nx, nz)
        if args.solver == "learned":
            p.cycle_correction = 3  # the headline's correction (the network is trained for 1024x256 inputs)
        sim = Simulation(p)
        sim.upload(state.initial_state(p, seed=1))
        row, q, dt = sim.step()
        print(json.dumps({"profile_step": True, "grid": [nx, nz], "tracers": int(sim.ntr), "cycles": q}), flush=True)
        sim.close()
        return
    if args.profile_shipped:
        from tracer_code_gb300 import Simulation, state
        p = shipped_params()
        sim = Simulation(p)
        sim.upload(state.initial_state(p, seed=1))
        out = []
        for _ in range(2):
            t0 = time.perf_counter()
            row, q, dt = sim.step()
            out.append({"cycles": q, "s": round(time.perf_counter() - t0, 4), "moved": (sim.equalize_row() or [0] * 5)[4]})
        print(json.dumps({"profile_shipped": True, "steps": out}), flush=True)
        sim.close()
        return
    if args.profile_solve:
        from tracer_code_gb300 import Simulation, state, learned
        p = workload_params("mixed" if args.solver == "learned" else args.solver)
        net = None
        if args.solver == "learned":
            p.learned_guess, p.cycle_correction = 3, 4
        sim = Simulation(p)
        if args.solver == "learned":
            net = learned.Net(1, p.nz, p.nx)
            net.load(GUESS_WEIGHTS)
            learned.attach(sim, net)
        sim.upload(state.initial_state(p, seed=1))
        n0 = Simulation.kernel_launches()
        q = sim.multigrid()
        print(json.dumps({"profile_solve": True, "solver": args.solver, "cycles": q, "launches_before_solve": n0,
                          "launches_in_solve": Simulation.kernel_launches() - n0}), flush=True)
        sim.close()
        if net:
            net.close()
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
