"""The learned pressure guess end to end, on held-out seeds.

A network is trained on the GPU by its own kernels on snapshots the solver
produces (rising drops at 32^3, training seeds 0-7, the first SIMPLE
iteration of 6 steps each), then attached to the mixed-precision solve of
held-out seeds 40 and 41.  The solve with the guess must reach the same
pressure tolerance every step (relative residual 1e-8 against ||f||) and the
same fields as the solve without it (relative L2 <= 1e-6, the bar of the
mixed form against FP64); the test prints what the guess gains -- pressure
iterations per step with and without it -- and requires that the trained
network beats the untrained one on the held-out snapshots and that the
guesses were kept (their residual below the zero guess's).
"""
import numpy as np
import pytest

from hydro_gb300 import capi
from tests.util import compare

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N = 32
STEPS = 6


def _run(seed, net=None):
    from hydro_gb300.net import attach, guess_stats
    from hydro_gb300.solver import Hydro
    from hydro_gb300.train_guess import RHO_SCALE, init_case, workload
    d, u0, q0, _ = workload(N, seed, "mixed")
    h = init_case(Hydro(d), d, u0, q0)
    if net is not None:
        attach(h, net, 1, RHO_SCALE)
    stats = [h.step() for _ in range(STEPS)]
    out = {"u": h.get_field(capi.F_VELOCITY), "p": h.get_field(capi.F_PRESSURE),
           "F": h.get_field(capi.F_VOLUME_FLUX), "q": h.get_field(capi.F_PARTIAL_DENSITY),
           "stats": stats}
    out["guess"] = guess_stats(h) if net is not None else (0, 0, 0)
    h.close()
    return out


def test_learned_guess_held_out(built):
    from hydro_gb300.net import Net
    from hydro_gb300.train_guess import snapshots, train
    net = Net((N, N, N), batch=4, seed=1)
    train_s = snapshots(net, N, range(8), STEPS)
    eval_s = snapshots(net, N, (40, 41), STEPS)
    loss0 = np.mean([net.eval_loss([s]) for s in eval_s])
    hist = train(net, train_s, 300, 4, 2e-3)
    loss1 = np.mean([net.eval_loss([s]) for s in eval_s])
    print("held-out loss %.4f -> %.4f (train loss %.4f -> %.4f)"
          % (loss0, loss1, np.mean(hist[:10]), np.mean(hist[-10:])))
    assert loss1 < 0.7 * loss0
    for seed in (40, 41):
        base = _run(seed)
        lrn = _run(seed, net)
        errs = compare(lrn, base)
        it_b = [s["pressure_iterations"] for s in base["stats"]]
        it_l = [s["pressure_iterations"] for s in lrn["stats"]]
        print("seed %d: pressure iterations per step without / with the guess %s / %s, "
              "guesses kept / dropped / skipped steps %s, field differences %s"
              % (seed, it_b, it_l, lrn["guess"], {k: "%.1e" % v for k, v in errs.items()}))
        assert all(v <= 1e-6 for v in errs.values()), errs
        for s in base["stats"] + lrn["stats"]:
            assert s["status"] == capi.OK and s["pressure_residual"] <= 1e-8
        used, dropped, skipped = lrn["guess"]
        # every step either tried the guess (kept or dropped) or skipped it
        # (back-off after a dropped guess)
        assert used + dropped + skipped == STEPS and used >= 1
    net.close()
