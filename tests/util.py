"""Shared helpers of the parity tests: run the same case on the GPU library
and on the CPU oracle and compare fields."""
import numpy as np

from hydro_gb300 import capi


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def demean(p):
    return p - p.mean()


def tight(d, omega_p=1.0):
    """Linear solves to machine-tight tolerance on both sides, so that a
    fixed number of SIMPLE iterations gives the same iterates."""
    d.velocity_tolerance = 1e-14
    d.velocity_iters_limit = 20000
    d.pressure_tolerance = 1e-13
    d.pressure_iters_limit = 20000
    return d


def run(solver, u0, q0, nsteps, heat=None):
    solver.set_field(capi.F_VELOCITY, u0)
    solver.set_field(capi.F_PARTIAL_DENSITY, q0)
    solver.init_state()
    if heat is not None:
        solver.heat_create(heat)
    stats = [solver.step() for _ in range(nsteps)]
    out = {
        "u": solver.get_field(capi.F_VELOCITY),
        "p": solver.get_field(capi.F_PRESSURE),
        "F": solver.get_field(capi.F_VOLUME_FLUX),
        "q": solver.get_field(capi.F_PARTIAL_DENSITY),
        "rho": solver.get_field(capi.F_DENSITY),
        "stats": stats,
    }
    if heat is not None:
        out["T"] = solver.temperature()
    return out


def compare(a, b, mask=None):
    """Relative L2 differences; the pressure up to its free constant, on
    the fluid cells (mask) when a rigid box excludes cells, whose pressure
    must then agree exactly."""
    if mask is None:
        dp = rel(demean(a["p"]), demean(b["p"]))
    else:
        dp = max(rel(demean(a["p"][mask]), demean(b["p"][mask])),
                 float(abs(a["p"][~mask] - b["p"][~mask]).max(initial=0.0)))
    out = {
        "u": rel(a["u"], b["u"]),
        "p": dp,
        "F": rel(a["F"], b["F"]),
        "q": rel(a["q"], b["q"]),
    }
    if "T" in a and "T" in b:
        out["T"] = rel(a["T"], b["T"])
    return out
