"""The graph-captured step (hydro_gpu_step_graph) against the host-driven
step (hydro_gpu_step): same kernels in the same order, so the fields agree
to rounding and the statistics (SIMPLE iterations, sweeps, pressure
iterations, substeps, dt) are identical.  The cases cover the plain FP64
path, the mixed path with both inner solvers, a SIMPLE loop stopped by its
tolerance (odd and even iteration counts), a pinned pressure cell, split
advection with surface tension, and auto dt (the graph is captured again
whenever dt changes)."""
import numpy as np
import pytest

from hydro_gb300 import capi, cases

from tests.util import compare

pytestmark = pytest.mark.gpu


def _run(d, u0, q0, nsteps, graph):
    from hydro_gb300.solver import Hydro
    h = Hydro(d)
    h.set_field(capi.F_VELOCITY, u0)
    h.set_field(capi.F_PARTIAL_DENSITY, q0)
    h.init_state()
    stats = [h.step_graph() if graph else h.step() for _ in range(nsteps)]
    return {
        "u": h.get_field(capi.F_VELOCITY),
        "p": h.get_field(capi.F_PRESSURE),
        "F": h.get_field(capi.F_VOLUME_FLUX),
        "q": h.get_field(capi.F_PARTIAL_DENSITY),
        "stats": stats,
        "time": h.time(),
    }


def _check(d, u0, q0, nsteps, tol=1e-12):
    a = _run(d, u0, q0, nsteps, graph=False)
    b = _run(d, u0, q0, nsteps, graph=True)
    errs = compare(b, a)
    assert all(v <= tol for v in errs.values()), errs
    keys = ("outer_iterations", "velocity_sweeps", "pressure_iterations",
            "advection_substeps", "dt", "dt_advection", "status")
    for sa, sb in zip(a["stats"], b["stats"]):
        for k in keys:
            assert sa[k] == sb[k], (k, sa, sb)
        assert sb["pressure_residual"] == pytest.approx(sa["pressure_residual"], rel=1e-9,
                                                        abs=1e-30)
        assert sb["convergence_indicator"] == pytest.approx(sa["convergence_indicator"],
                                                            rel=1e-9)
    assert a["time"] == pytest.approx(b["time"], rel=1e-15)
    return a, b


def test_graph_step_cavity_fp64_converged(built):
    """FP64, SIMPLE loop to a tolerance: iteration counts vary per step."""
    d, u0, q0 = cases.cavity(n=24, mu=0.01, dt=5e-3)
    d.convergence_tolerance = 1e-4
    d.num_iterations_limit = 9
    d.pressure_fixed_cell = 5
    a, _ = _check(d, u0, q0, 4)
    its = {s["outer_iterations"] for s in a["stats"]}
    assert len(its) > 1 or its & {1, 3, 5, 7, 9}, its


def test_graph_step_drops_mixed_mgcg(built):
    d, u0, q0, _ = cases.rising_drops(n=16, seed=3, dt_max=5e-3)
    d.precision = capi.MIXED
    d.pressure_solver = capi.LINEAR_MGCG
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 3
    d.pressure_tolerance = 1e-9
    _check(d, u0, q0, 3)


def test_graph_step_drops_mixed_jacobi_cg(built):
    d, u0, q0, _ = cases.rising_drops(n=12, seed=4, dt_max=5e-3)
    d.precision = capi.MIXED
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 2
    d.pressure_tolerance = 1e-9
    _check(d, u0, q0, 2)


def test_graph_step_dam_split_sigma_auto_dt(built):
    d, u0, q0 = cases.broken_dam(nx=40, ny=20, dt_auto=True, cfl=0.5, dt_max=5e-4)
    d.tvd_split = 1
    d.sigma = 0.05
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 4
    _check(d, u0, q0, 3)


def test_graph_step_multigrid_grid_levels(built):
    """Grid-launched and in-CTA multigrid levels inside graph WHILE nodes."""
    d, u0, q0, _ = cases.rising_drops(n=32, seed=1, dt_max=4e-3)
    d.precision = capi.MIXED
    d.pressure_solver = capi.LINEAR_MGCG
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 2
    _check(d, u0, q0, 2)


def test_graph_step_simpler_channel(built):
    """SIMPLER's second pressure solve and the outlet rebalancing inside the
    graph-captured loops."""
    d, u0, q0 = cases.channel(nx=20, ny=10, dt=1e-2)
    d.simpler = 1
    d.pressure_fixed_cell = 3
    d.convergence_tolerance = 1e-5
    d.num_iterations_limit = 7
    _check(d, u0, q0, 3)


@pytest.mark.parametrize("pattern", ["HGHG", "GHGH", "GGHHG"])
def test_graph_and_host_steps_interleaved(built, pattern):
    """Host-driven and graph-captured steps interleaved on one context give
    the host-only run: a host step rotates the time and iteration layers
    (pointer swaps), after which the graph is captured again instead of
    replaying launches on the layers it was captured on."""
    from hydro_gb300.solver import Hydro
    d, u0, q0 = cases.cavity(n=32, mu=1e-3, dt=1e-3)
    d.precision = capi.MIXED
    d.pressure_solver = capi.LINEAR_MGCG
    ref = _run(d, u0, q0, len(pattern), graph=False)
    h = Hydro(d)
    h.set_field(capi.F_VELOCITY, u0)
    h.set_field(capi.F_PARTIAL_DENSITY, q0)
    h.init_state()
    for ch in pattern:
        st = h.step_graph() if ch == "G" else h.step()
        assert st["status"] == capi.OK
    got = {"u": h.get_field(capi.F_VELOCITY), "p": h.get_field(capi.F_PRESSURE),
           "F": h.get_field(capi.F_VOLUME_FLUX), "q": h.get_field(capi.F_PARTIAL_DENSITY)}
    errs = compare(got, {k: ref[k] for k in got})
    assert all(v <= 1e-12 for v in errs.values()), errs


def test_graph_launch_counts(built):
    """Kernels counted for graph launches (the captured bodies count their
    runs on the device): a batch step runs exactly the kernels of its cases'
    graph steps run alone."""
    from hydro_gb300.solver import Batch, Hydro, launch_count
    specs = [cases.cavity(n=n, mu=1.0 / re, dt=1e-3) for n, re in ((32, 100), (48, 1000), (64, 400))]
    descs = []
    for d, _, _ in specs:
        d = d.copy()
        d.precision = capi.MIXED
        d.pressure_solver = capi.LINEAR_MGCG
        descs.append(d)
    alone = []
    for d, (_, u0, q0) in zip(descs, specs):
        h = Hydro(d)
        h.set_field(capi.F_VELOCITY, u0)
        h.set_field(capi.F_PARTIAL_DENSITY, q0)
        h.init_state()
        h.step_graph()  # capture
        c0 = launch_count()
        st = h.step_graph()
        alone.append((launch_count() - c0, st["outer_iterations"]))
        h.close()
    b = Batch(descs)
    for c, (_, u0, q0) in zip(b.cases, specs):
        c.set_field(capi.F_VELOCITY, u0)
        c.set_field(capi.F_PARTIAL_DENSITY, q0)
    b.init_state()
    b.step()  # capture
    c0 = launch_count()
    b.step()
    got = launch_count() - c0
    b.close()
    assert all(n > 0 for n, _ in alone), alone
    assert got == sum(n for n, _ in alone), (got, alone)
