"""Generate training samples for the learned multigrid guess and train it.

    python -m tracer_code_gb300.train_guess [--samples 5000] [--steps 3000]
        [--out tracer_code_gb300/weights/guess_512x128.npy]

Samples: every multigrid solve of short runs of the 1024x256 case's setup on
a 512x128 grid (25 tracers per cell replaced by 4 to save time; the solve
does not depend on the tracer count beyond the composition field), each run
with its own seed and physics drawn log-uniformly from viscosity contrast
1e2..1e5 and Ra 1e6..1e7, and uniformly from B 0.3..1.0.  The solver is the
mixed-precision multigrid without the guess, iterating to the same 1e-8
relative residual, so each sample's target is the converged streamfunction.
A solve's sample is (log10 viscosity, RHS, previous streamfunction) -> new
streamfunction (include/tracer_nn.h).  Solves that start from a zero
streamfunction (the first of a run) carry no previous field and are dropped.

Training: the library's own kernels (BF16 tcgen05 convolutions, FP32 Adam),
batches of 8, cosine learning-rate decay; 5 % of the samples held out.
Writes the parameters (float16) and a JSON summary next to them.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np


def sample_params(rng, nx, nz):
    from .abi import config_1024x256
    p = config_1024x256()
    p.nx, p.nz, p.tpc, p.grids = nx, nz, 4, 5
    ra = 10.0 ** rng.uniform(6.0, 7.0)
    b = rng.uniform(0.3, 1.0)
    p.RaT = ra
    p.RaC[0] = b * ra
    p.visT = 10.0 ** rng.uniform(2.0, 5.0)
    p.mg_zero_coarse = 1
    p.solver_precision = 1
    return p, {"Ra": ra, "B": b, "visT": p.visT}


def generate(n_samples: int, nx: int, nz: int, steps_per_run: int, seed: int, log=print):
    import torch
    from . import Simulation, TracerError, state
    from . import learned
    H, W = nz, nx
    raw = torch.empty((n_samples, 3, H, W), dtype=torch.float32, device="cuda")
    sf = torch.empty((n_samples, H, W), dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(seed)
    count, run = 0, 0
    runs = []
    t0 = time.time()
    while count < n_samples:
        p, phys = sample_params(rng, nx, nz)
        sim = Simulation(p)
        sim.upload(state.initial_state(p, seed=1000 + run))
        learned.record_solves(sim, raw.data_ptr() + count * 3 * H * W * 4, sf.data_ptr() + count * H * W * 4,
                              n_samples - count)
        done = 0
        try:
            for _ in range(steps_per_run):
                sim.step()
                done += 1
        except TracerError as e:
            phys["stopped"] = str(e)
        got = learned.record_count(sim)
        sim.close()
        count += got
        phys.update({"steps": done, "samples": got})
        runs.append(phys)
        run += 1
        log(f"run {run}: {phys} total {count} ({time.time() - t0:.0f} s)")
    return raw, sf, runs


def train(raw, sf, steps: int, batch: int, lr: float, seed: int, log=print):
    import torch
    from .learned import Net
    n, _, H, W = raw.shape
    rms_prev = raw[:, 2].pow(2).mean(dim=(1, 2)).sqrt()
    rms_new = sf.pow(2).mean(dim=(1, 2)).sqrt()
    keep = torch.nonzero(rms_prev > 1e-3 * rms_new).flatten()
    g = torch.Generator(device="cpu").manual_seed(seed)
    perm = keep[torch.randperm(keep.numel(), generator=g).to(keep.device)]
    n_val = max(1, perm.numel() // 20)
    val, tr = perm[:n_val], perm[n_val:]
    net = Net(batch, H, W, seed=seed)
    xb = torch.empty((batch, 3, H, W), dtype=torch.float32, device="cuda")
    yb = torch.empty((batch, H, W), dtype=torch.float32, device="cuda")

    def val_loss():
        tot, m = 0.0, 0
        for j in range(0, val.numel() - batch + 1, batch):
            idx = val[j:j + batch]
            torch.index_select(raw, 0, idx, out=xb)
            torch.index_select(sf, 0, idx, out=yb)
            tot += net.loss_backward(xb.data_ptr(), yb.data_ptr(), batch)
            m += 1
        return tot / max(m, 1)

    hist = []
    v0 = val_loss()
    t0 = time.time()
    for it in range(steps):
        idx = tr[torch.randint(0, tr.numel(), (batch,), generator=g).to(tr.device)]
        torch.index_select(raw, 0, idx, out=xb)
        torch.index_select(sf, 0, idx, out=yb)
        loss = net.loss_backward(xb.data_ptr(), yb.data_ptr(), batch)
        a = lr * (0.01 + 0.99 * 0.5 * (1.0 + math.cos(math.pi * it / steps)))
        net.adam(a)
        if it % 250 == 0 or it == steps - 1:
            hist.append({"step": it, "train": loss, "lr": a})
            log(f"step {it}: loss {loss:.4e} lr {a:.2e} ({time.time() - t0:.0f} s)")
    v1 = val_loss()
    return net, {"kept": int(keep.numel()), "train": int(tr.numel()), "val": int(val.numel()),
                 "val_loss_init": v0, "val_loss_final": v1, "history": hist, "train_s": time.time() - t0}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=5000)
    ap.add_argument("--steps-per-run", type=int, default=30)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--nz", type=int, default=128)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(__file__), "weights", "guess_512x128.npy"))
    args = ap.parse_args()
    t0 = time.time()
    raw, sf, runs = generate(args.samples, args.nx, args.nz, args.steps_per_run, args.seed)
    tg = time.time() - t0
    net, info = train(raw, sf, args.steps, args.batch, args.lr, args.seed)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.save(args.out, net.get_params().astype(np.float16))
    info.update({"samples": args.samples, "grid": f"{args.nx}x{args.nz}", "runs": runs, "generate_s": tg,
                 "steps": args.steps, "batch": args.batch, "lr": args.lr})
    with open(os.path.splitext(args.out)[0] + ".json", "w") as f:
        json.dump(info, f, indent=1)
    print(json.dumps({k: v for k, v in info.items() if k not in ("runs", "history")}))


if __name__ == "__main__":
    main()
