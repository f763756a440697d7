"""Batched cases (hydro_gpu_batch_*): every case of a batch advanced by one
graph launch per batch step gives the same fields and statistics as the
same case stepped alone by hydro_gpu_step.  Cases of uneven size and
configuration share a batch (the lid-driven cavities of many independent
cases at reduced sizes, plus a mixed-precision multigrid case and a
two-phase case with advection and auto dt)."""
import pytest

from hydro_gb300 import capi, cases

from tests.util import compare

pytestmark = pytest.mark.gpu

KEYS = ("outer_iterations", "velocity_sweeps", "pressure_iterations", "advection_substeps",
        "dt", "dt_advection", "status")


def _alone(d, u0, q0, nsteps):
    from hydro_gb300.solver import Hydro
    h = Hydro(d)
    h.set_field(capi.F_VELOCITY, u0)
    h.set_field(capi.F_PARTIAL_DENSITY, q0)
    h.init_state()
    stats = [h.step() for _ in range(nsteps)]
    return _fields(h), stats


def _fields(h):
    return {"u": h.get_field(capi.F_VELOCITY), "p": h.get_field(capi.F_PRESSURE),
            "F": h.get_field(capi.F_VOLUME_FLUX), "q": h.get_field(capi.F_PARTIAL_DENSITY)}


def _batch_cases():
    out = [(d, u0, q0) for d, u0, q0, _ in
           cases.cavity_batch(ncases=6, seed=11, sizes=(12, 16, 20, 24, 32), dt=1e-3)]
    d, u0, q0, _ = cases.rising_drops(n=16, seed=2, dt_max=5e-3)
    d.precision = capi.MIXED
    d.pressure_solver = capi.LINEAR_MGCG
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 2
    out.append((d, u0, q0))
    d, u0, q0 = cases.broken_dam(nx=32, ny=16, dt_auto=True, dt_max=5e-4, smooth_times=2)
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 3
    out.append((d, u0, q0))
    return out


def test_batch_matches_cases_stepped_alone(built):
    from hydro_gb300.solver import Batch
    specs = _batch_cases()
    nsteps = 3
    b = Batch([d for d, _, _ in specs])
    for c, (d, u0, q0) in zip(b.cases, specs):
        c.set_field(capi.F_VELOCITY, u0)
        c.set_field(capi.F_PARTIAL_DENSITY, q0)
    b.init_state()
    bstats = [b.step() for _ in range(nsteps)]
    for i, (d, u0, q0) in enumerate(specs):
        ref, rstats = _alone(d, u0, q0, nsteps)
        errs = compare(_fields(b.cases[i]), ref)
        assert all(v <= 1e-12 for v in errs.values()), (i, errs)
        for step in range(nsteps):
            sa, sb = rstats[step], bstats[step][i]
            for k in KEYS:
                assert sa[k] == sb[k], (i, step, k, sa, sb)
    b.close()
