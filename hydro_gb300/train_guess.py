"""Train the learned pressure guess on snapshots the solver produces.

    python -m hydro_gb300.train_guess --n 192 --seeds 0-39 --steps 100 \\
        --iters 4000 --batch 4 --out weights.npy

For every training seed a rising-drops case (cases.rising_drops: unit cube,
ambient rho 10, drops rho 1, mu 1e-2, g = -1 along z) starts at rest in
hydrostatic balance and runs `--steps` time steps with the FP64 kernels and
the multigrid-preconditioned FP64 refinement solve; the first SIMPLE
iteration's pressure system of every step -- right-hand side f, density,
converged p' -- is packed into a BF16 sample kept on the device.  The network
(include/hydro_net.h) is then trained by its own forward / backward / Adam
kernels on random batches of the samples.  The script prints the loss and
writes the parameters (numpy float32) to --out.  Samples at 192^3 take 42 MB
each: 4000 of them (40 seeds x 100 steps) fit in the 280 GB of one GB300.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

from . import capi, cases
from .net import Net, snapshot_step
from .solver import Hydro

RHO_SCALE = 0.1  # density input: rho / 10 (the ambient density of the workload)


def workload(n, seed, precision="fp64", outer=5):
    """The rising-drops workload at n^3 (the benchmark's settings)."""
    d, u0, q0, drops = cases.rising_drops(n=n, seed=seed, dt_max=2e-3)
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = outer
    d.velocity_solver = capi.LINEAR_GAUSS_SEIDEL
    d.velocity_tolerance = 1e-8
    d.velocity_iters_limit = 200
    d.pressure_tolerance = 1e-8
    d.pressure_iters_limit = 20000
    d.precision = capi.MIXED if precision == "mixed" else capi.FP64
    d.pressure_solver = capi.LINEAR_MGCG
    return d, u0, q0, drops


def init_case(h, d, u0, q0):
    """Rest, partial densities, hydrostatic pressure (both time layers)."""
    h.set_field(capi.F_VELOCITY, u0)
    h.set_field(capi.F_PARTIAL_DENSITY, q0)
    h.init_state()
    p0 = cases.hydrostatic_pressure(d, h.get_field(capi.F_DENSITY))
    for layer in (capi.TIME_CURR, capi.TIME_PREV):
        h.set_field(capi.F_PRESSURE, p0, layer)
    return h


def snapshots(net, n, seeds, steps, precision="fp64", log=None):
    """Packed samples (torch uint8 device tensors) of the first SIMPLE
    iteration of `steps` steps of every seed."""
    import torch
    out = []
    for seed in seeds:
        d, u0, q0, _ = workload(n, seed, precision)
        h = init_case(Hydro(d), d, u0, q0)
        for _ in range(steps):
            buf = torch.empty(net.sample_bytes, dtype=torch.uint8, device="cuda")
            snapshot_step(h, net, RHO_SCALE, buf.data_ptr())
            out.append(buf)
        h.close()
        if log:
            log("seed %d: %d samples" % (seed, len(out)))
    return out


def train(net, samples, iters, batch, lr, seed=0, log=None, lr_final=None):
    """Adam on random batches; cosine decay of the learning rate to
    lr_final.  Returns the loss history (one value per step)."""
    rng = np.random.default_rng(seed)
    lr_final = lr * 0.05 if lr_final is None else lr_final
    hist = []
    for it in range(iters):
        idx = rng.choice(len(samples), size=min(batch, len(samples)), replace=False)
        a = lr_final + 0.5 * (lr - lr_final) * (1.0 + np.cos(np.pi * it / max(iters, 1)))
        hist.append(net.train_step([samples[i] for i in idx], a))
        if log and (it % 200 == 0 or it == iters - 1):
            log("iter %d loss %.5f lr %.2e" % (it, hist[-1], a))
    return hist


def _range(text):
    out = []
    for part in text.split(","):
        if "-" in part:
            a, b = part.split("-")
            out.extend(range(int(a), int(b) + 1))
        else:
            out.append(int(part))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--n", type=int, default=192)
    ap.add_argument("--seeds", default="0-39")
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--iters", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval-seeds", default="40-41")
    ap.add_argument("--eval-steps", type=int, default=5)
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    import torch
    t0 = time.time()
    log = lambda m: print("[%.0f s] %s" % (time.time() - t0, m), flush=True)  # noqa: E731
    net = Net((a.n, a.n, a.n), batch=a.batch, seed=1)
    train_s = snapshots(net, a.n, _range(a.seeds), a.steps, log=log)
    eval_s = snapshots(net, a.n, _range(a.eval_seeds), a.eval_steps, log=log)
    loss0 = np.mean([net.eval_loss([s]) for s in eval_s])
    log("held-out loss before training %.5f" % loss0)
    torch.cuda.synchronize()
    t1 = time.time()
    hist = train(net, train_s, a.iters, a.batch, a.lr, log=log)
    torch.cuda.synchronize()
    t_train = time.time() - t1
    loss1 = np.mean([net.eval_loss([s]) for s in eval_s])
    log("held-out loss after training %.5f (%d steps in %.1f s)" % (loss1, a.iters, t_train))
    net.save(a.out)
    meta = {"n": a.n, "seeds": a.seeds, "steps": a.steps, "samples": len(train_s),
            "iters": a.iters, "batch": a.batch, "lr": a.lr, "rho_scale": RHO_SCALE,
            "train_seconds": round(t_train, 1), "heldout_loss_before": float(loss0),
            "heldout_loss_after": float(loss1), "train_loss_last": float(np.mean(hist[-50:]))}
    with open(os.path.splitext(a.out)[0] + ".json", "w") as f:
        json.dump(meta, f, indent=1)
    log(json.dumps(meta))
    return 0


if __name__ == "__main__":
    sys.exit(main())
