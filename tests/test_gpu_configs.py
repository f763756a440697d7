"""The five configurations of the workload at their full sizes, through
properties that do not depend on size: the plain FP64 path against the
oracle where the oracle finishes in seconds (the 64^2 cavity over its 200
steps, the 512x256 breaking dam over ten steps), the mixed forms against
the FP64 path at 8.4 M and 7.1 M cells over 50 steps, conservation of every
phase over many steps, and the 512-case batch against its cases stepped
alone."""
import numpy as np
import pytest

from hydro_gb300 import capi, cases
from tests.util import compare, rel, run, tight

pytestmark = pytest.mark.gpu


def _pinned(d, iters):
    d.convergence_tolerance, d.num_iterations_limit = 0.0, iters
    return d


def test_c1_cavity_64_over_200_steps_vs_oracle(built):
    """Lid-driven cavity, 64^2, Re 100, dt 1e-3, 200 steps (outer iterations
    pinned at 2 per step for the comparison)."""
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    d, u0, q0 = cases.cavity(n=64, mu=0.01, dt=1e-3)
    _pinned(tight(d), 2)
    a = run(Hydro(d), u0, q0, 200)
    do = d.copy()
    do.pressure_solver = capi.LINEAR_CG
    b = run(Oracle(do, threads=8), u0, q0, 200)
    errs = compare(a, b)
    assert all(v <= 1e-10 for v in errs.values()), errs
    assert np.abs(a["u"]).max() > 0.5  # the lid drove the flow


def _fields(s):
    return {"u": s.get_field(capi.F_VELOCITY), "p": s.get_field(capi.F_PRESSURE),
            "F": s.get_field(capi.F_VOLUME_FLUX), "q": s.get_field(capi.F_PARTIAL_DENSITY)}


def test_c2_dam_512x256_vs_oracle_and_conservation(built):
    """Breaking dam at 512x256: ten steps against the oracle, compared after
    every step (the errors stay at rounding level, they do not grow), then
    15 steps of the mixed form conserving the partial mass of both phases.
    (With the example scripts' smoothing; at this resolution and the default
    loose velocity tolerance the SIMPLE loop stops converging after ~20 steps
    and the run diverges near step 27 identically in FP64 and mixed
    precision, as the reference algorithm does in the oracle.)"""
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    d, u0, q0 = cases.broken_dam(nx=512, ny=256, dt_auto=True, dt_max=1e-3, smooth_times=2)
    _pinned(tight(d, 1.0), 2)
    d.pressure_tolerance = 1e-12
    do = d.copy()
    do.pressure_solver = capi.LINEAR_CG
    a, b = Hydro(d), Oracle(do, threads=16)
    run(a, u0, q0, 0)
    run(b, u0, q0, 0)
    history = []
    for step in range(10):
        sa, sb = a.step(), b.step()
        assert sa["outer_iterations"] == sb["outer_iterations"]
        assert sa["dt"] == pytest.approx(sb["dt"], rel=1e-12)
        errs = compare(_fields(a), _fields(b))
        history.append(max(errs.values()))
        assert all(v <= 1e-9 for v in errs.values()), (step, errs)
    print("C2 per-step max relative error vs oracle:", ["%.1e" % e for e in history])
    d2, u0, q0 = cases.broken_dam(nx=512, ny=256, dt_auto=True, dt_max=1e-3, smooth_times=2)
    d2.precision = capi.MIXED
    d2.pressure_solver = capi.LINEAR_MGCG
    h = Hydro(d2)
    run(h, u0, q0, 0)
    m0 = h.calc_stat()
    stats = [h.step() for _ in range(15)]
    m1 = h.calc_stat()
    assert all(s["status"] == 0 for s in stats), [
        (i, s["status"], s["pressure_residual"], s["pressure_iterations"],
         s["pressure_unconverged"]) for i, s in enumerate(stats) if s["status"] != 0]
    for i in range(2):
        assert abs(m1.partial_mass[i] - m0.partial_mass[i]) <= 1e-11 * abs(m0.partial_mass[i])
    q = h.get_field(capi.F_PARTIAL_DENSITY)
    assert np.all(np.isfinite(q))


@pytest.mark.parametrize("config", ["c3_rt_128x128x512", "c4_drops_192"])
def test_mixed_forms_vs_fp64_full_size(built, config):
    """Mixed precision with the multigrid CG against the FP64 path (FP64
    kernels, multigrid-preconditioned refinement) at full size over 50 steps
    of 3 SIMPLE iterations, compared after every step: every field --
    velocity, pressure (up to its constant), fluxes, partial densities --
    within 1e-6 relative L2 at every step, every pressure solve at its
    tolerance.  (Measured: u <= 3.2e-7, p <= 3.1e-9 over 30 steps at 192^3;
    u <= 5.6e-7, p <= 1.3e-9 for Rayleigh-Taylor; the velocity error grows
    by about 1e-8 a step.)"""
    from hydro_gb300.solver import Hydro
    if config.startswith("c3"):
        d, u0, q0 = cases.rayleigh_taylor(seed=0)[:3]
    else:
        d, u0, q0, _ = cases.rising_drops(n=192, seed=0, dt_max=2e-3)
    _pinned(d, 3)
    d.velocity_tolerance, d.velocity_iters_limit = 1e-10, 400
    d.pressure_tolerance, d.pressure_iters_limit = 1e-10, 20000
    d.precision = capi.FP64
    d.pressure_solver = capi.LINEAR_MGCG
    dm = d.copy()
    dm.precision = capi.MIXED
    a, b = Hydro(d), Hydro(dm)
    run(a, u0, q0, 0)
    run(b, u0, q0, 0)
    worst = {}
    for step in range(50):
        sa, sb = a.step(), b.step()
        for s in (sa, sb):
            assert s["status"] == 0 and s["pressure_residual"] <= 1e-10
        errs = compare(_fields(b), _fields(a))
        for k, v in errs.items():
            worst[k] = max(worst.get(k, 0.0), v)
        assert all(v <= 1e-6 for v in errs.values()), (step, errs)
    print(config, "largest relative error over 50 steps:", {k: "%.1e" % v for k, v in worst.items()})


@pytest.mark.parametrize("cta_threads,cta_cluster", [(0, 0), (512, 1), (1024, 4)])
def test_c5_batch_512_cavities(built, cta_threads, cta_cluster):
    """512 cavities of 64^2..256^2 (13.4 M cells) in one batch, mixed with the
    multigrid CG, SIMPLE converged per case: two batch steps, and four cases
    of every size stepped alone give the same fields -- with grid-wide
    solver launches, with every linear solve by one CTA of 512 threads, and
    by one cluster of four CTAs of 1024 threads."""
    from hydro_gb300.solver import Batch, Hydro
    specs = cases.cavity_batch(ncases=512, seed=0)
    descs = []
    for d, u0, q0, _ in specs:
        d = d.copy()
        d.precision = capi.MIXED
        d.pressure_solver = capi.LINEAR_MGCG
        d.cta_threads = cta_threads
        d.cta_cluster = cta_cluster
        descs.append(d)
    b = Batch(descs)
    for c, (d, u0, q0, _) in zip(b.cases, specs):
        c.set_field(capi.F_VELOCITY, u0)
        c.set_field(capi.F_PARTIAL_DENSITY, q0)
    b.init_state()
    st = [b.step() for _ in range(2)]
    assert all(s["status"] == 0 for step in st for s in step)
    picked = {}
    for i, d in enumerate(descs):
        picked.setdefault(d.n[0], [])
        if len(picked[d.n[0]]) < 4:
            picked[d.n[0]].append(i)
    for n, idx in picked.items():
        for i in idx:
            d, u0, q0, _ = specs[i]
            alone = run(Hydro(descs[i]), u0, q0, 2)
            u = b.cases[i].get_field(capi.F_VELOCITY)
            assert rel(u, alone["u"]) <= 1e-12, (n, i)


@pytest.mark.parametrize("n,threads,cluster",
                         [(64, 256, 1), (96, 512, 1), (256, 1024, 1), (96, 1024, 4),
                          (256, 1024, 8)])
def test_cta_solvers_match_grid_solvers(built, n, threads, cluster):
    """The one-CTA (or one-cluster) linear solves against the grid-wide ones on a cavity
    (Re 1000, mixed, multigrid CG), host-driven and graph-captured steps
    interleaved: velocity and pressure within 1e-6 of the run's scale after
    5 steps of 5 SIMPLE iterations (both solve to a pressure residual of
    1e-10 and a velocity update of 1e-7; only the summation order differs),
    and every pressure solve converged."""
    from hydro_gb300.solver import Hydro
    d, u0, q0 = cases.cavity(n=n, mu=1e-3, dt=1e-3)
    _pinned(d, 5)
    d.precision = capi.MIXED
    d.pressure_solver = capi.LINEAR_MGCG
    d.pressure_tolerance = 1e-10
    d.velocity_tolerance = 1e-7
    dc = d.copy()
    dc.cta_threads = threads
    dc.cta_cluster = cluster
    a, b = Hydro(d), Hydro(dc)
    for h in (a, b):
        h.set_field(capi.F_VELOCITY, u0)
        h.set_field(capi.F_PARTIAL_DENSITY, q0)
        h.init_state()
    for step in range(5):
        sa = a.step()
        sb = b.step_graph() if step % 2 else b.step()
        assert sa["status"] == 0 and sb["status"] == 0, (sa, sb)
        assert sb["pressure_unconverged"] == 0
    ua, ub = a.get_field(capi.F_VELOCITY), b.get_field(capi.F_VELOCITY)
    pa, pb = a.get_field(capi.F_PRESSURE), b.get_field(capi.F_PRESSURE)
    assert np.abs(ua - ub).max() <= 1e-6 * np.abs(ua).max(), np.abs(ua - ub).max()
    assert np.abs(pa - pb).max() <= 1e-6 * np.abs(pa).max(), np.abs(pa - pb).max()


def test_cta_solvers_limits_and_nan(built):
    """The one-CTA pressure solve reports a pressure iteration limit as
    HYDRO_NOT_CONVERGED (host-driven and graph-captured) and a NaN in the
    system as HYDRO_ERR_NAN; a rigid box or a periodic direction with
    cta_threads set is refused."""
    from hydro_gb300.solver import Hydro, make
    d, u0, q0 = cases.cavity(n=64, mu=1e-2, dt=1e-3)
    d.precision = capi.MIXED
    d.pressure_solver = capi.LINEAR_MGCG
    d.cta_threads = 256
    d.pressure_tolerance, d.pressure_iters_limit = 1e-12, 1
    for graph in (False, True):
        h = make(d, u0, q0)
        st = h.step_graph() if graph else h.step()
        assert st["status"] == capi.NOT_CONVERGED and st["pressure_unconverged"] >= 1, st
        assert np.all(np.isfinite(h.get_field(capi.F_PRESSURE)))
    d.pressure_iters_limit = 20000
    h = make(d, u0, q0)
    assert h.step()["status"] == capi.OK
    u = h.get_field(capi.F_VELOCITY)
    u[d.ncells // 2] = np.nan
    h.set_field(capi.F_VELOCITY, u)
    with pytest.raises(capi.HydroError) as e:
        h.step()
    assert e.value.status == capi.ERR_NAN
    bad = d.copy()
    bad.periodic[0] = 1
    with pytest.raises(capi.HydroError) as e:
        Hydro(bad)
    assert e.value.status == capi.ERR_UNSUPPORTED
