"""GPU parity: libhydro_gpu.so (CUDA, sm_103a) against the CPU oracle on the
same seeded inputs.  Linear solves are tight on both sides and the number of
SIMPLE iterations per step is pinned, so iterates must agree to rounding:
velocity, pressure (up to its free constant), fluxes and partial densities
to relative L2 <= 1e-10 (the tolerance of the FP64 drop-in)."""
import numpy as np
import pytest

from hydro_gb300 import capi, cases
from tests.util import compare, rel, run, tight

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _pair(d, u0, q0, nsteps):
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    g = run(Hydro(d), u0, q0, nsteps)
    do = d.copy()
    do.velocity_solver = capi.LINEAR_GAUSS_SEIDEL
    do.pressure_solver = capi.LINEAR_CG
    o = run(Oracle(do), u0, q0, nsteps)
    return g, o


def _check(g, o, tol=TOL):
    errs = compare(g, o)
    assert all(v <= tol for v in errs.values()), errs
    for sg, so in zip(g["stats"], o["stats"]):
        assert sg["outer_iterations"] == so["outer_iterations"]
        assert sg["advection_substeps"] == so["advection_substeps"]
        assert abs(sg["dt"] - so["dt"]) <= 1e-12 * so["dt"]
    return errs


def test_cavity_2d(built):
    d, u0, q0 = cases.cavity(n=16, mu=0.01, dt=1e-2)
    tight(d)
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 3
    g, o = _pair(d, u0, q0, 3)
    _check(g, o)


def test_cavity_2d_nonsquare_pinned(built):
    d, u0, q0 = cases.cavity(n=12, mu=0.02, dt=5e-3)
    d.n[0], d.n[1] = 20, 12
    d.hi[0] = 1.7
    u0 = np.zeros(d.ncells * 2)
    q0 = np.ones(d.ncells)
    d.pressure_fixed_cell = 37
    d.pressure_fixed_value = 0.0
    d.guess_extrapolation = 0.5
    d.velocity_relaxation_factor = 0.7
    tight(d)
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 4
    g, o = _pair(d, u0, q0, 3)
    _check(g, o)


def test_broken_dam_2d_advection(built):
    d, u0, q0 = cases.broken_dam(nx=40, ny=20, dt_auto=True, dt_max=5e-4, smooth_times=2)
    tight(d)
    d.convergence_tolerance = 1e-7
    d.num_iterations_limit = 40
    g, o = _pair(d, u0, q0, 3)
    _check(g, o, tol=1e-9)


def test_broken_dam_split_sigma(built):
    d, u0, q0 = cases.broken_dam(nx=24, ny=12, dt_auto=False, dt=1e-3, smooth_times=1)
    tight(d)
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 2
    d.tvd_split = 1
    d.sigma = 0.05
    d.force_geometric_average = 1
    g, o = _pair(d, u0, q0, 2)
    _check(g, o)


def test_rising_drops_3d(built):
    d, u0, q0, _ = cases.rising_drops(n=12, seed=3, dt_max=5e-3)
    tight(d)
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 3
    g, o = _pair(d, u0, q0, 2)
    _check(g, o)


def test_cavity_3d_first_order_time(built):
    d, u0, q0 = cases.cavity(n=10, dim=3, dt=1e-2)
    d.n[2] = 7
    u0 = np.zeros(d.ncells * 3)
    q0 = np.ones(d.ncells)
    d.time_second_order = 0
    tight(d)
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 3
    g, o = _pair(d, u0, q0, 2)
    _check(g, o)


def test_mixed_precision_matches_fp64(built):
    from hydro_gb300.solver import Hydro
    d, u0, q0, _ = cases.rising_drops(n=16, seed=5, dt_max=5e-3)
    d.pressure_tolerance = 1e-10
    d.velocity_tolerance = 1e-12
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 4
    a = run(Hydro(d), u0, q0, 3)
    dm = d.copy()
    dm.precision = capi.MIXED
    b = run(Hydro(dm), u0, q0, 3)
    errs = compare(b, a)
    assert all(v <= 1e-6 for v in errs.values()), errs
    for s in b["stats"]:
        assert s["pressure_residual"] <= 1e-10


@pytest.mark.parametrize("shape", [(16, 16, 16), (24, 16, 8), (20, 12, 10), (32, 32, 16),
                                   (48, 32, 24)])
def test_multigrid_cg_matches_fp64(built, shape):
    """Mixed precision with the multigrid-preconditioned CG: same fields as
    the FP64 Jacobi-CG path within the mixed tolerance, pressure residual
    reached, few iterations (power-of-two and non-power-of-two blocks; the
    first three run the whole V-cycle inside one CTA, the last two have one
    and two grid levels above the in-CTA levels)."""
    from hydro_gb300.solver import Hydro
    d, u0, q0, _ = cases.rising_drops(n=16, seed=5, dt_max=5e-3)
    d.n[0], d.n[1], d.n[2] = shape
    d.hi[0], d.hi[1], d.hi[2] = shape[0] / 16.0, shape[1] / 16.0, shape[2] / 16.0
    from hydro_gb300.cases import cell_centers, two_phase_q
    x, y, z = cell_centers(d)
    alpha1 = (((x - 0.4) ** 2 + (y - 0.3) ** 2 + (z - 0.25) ** 2) < 0.15 ** 2).astype(float)
    q0 = two_phase_q(d, alpha1, 2)
    u0 = np.zeros(d.ncells * 3)
    d.pressure_tolerance = 1e-10
    d.velocity_tolerance = 1e-12
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = 3
    a = run(Hydro(d), u0, q0, 3)
    dm = d.copy()
    dm.precision = capi.MIXED
    dm.pressure_solver = capi.LINEAR_MGCG
    b = run(Hydro(dm), u0, q0, 3)
    errs = compare(b, a)
    assert all(v <= 1e-6 for v in errs.values()), errs
    for sa, sb in zip(a["stats"], b["stats"]):
        assert sb["pressure_residual"] <= 1e-10
        assert sb["pressure_iterations"] < sa["pressure_iterations"]


def test_fp64_multigrid_refinement_matches_oracle(built):
    """The FP64 path with the multigrid-preconditioned pressure solve (FP32
    V-cycle + CG inside FP64 iterative refinement): the FP64 system solved
    to the FP64 tolerance, so the same fields as the oracle to 1e-10, in a
    fraction of the Jacobi-CG iterations; the graph-captured step agrees."""
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    d, u0, q0, _ = cases.rising_drops(n=16, seed=3, dt_max=5e-3)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.pressure_solver = capi.LINEAR_MGCG
    a = run(Hydro(d), u0, q0, 3)
    do = d.copy()
    do.pressure_solver = capi.LINEAR_CG
    b = run(Oracle(do), u0, q0, 3)
    errs = compare(a, b)
    assert all(v <= 1e-10 for v in errs.values()), errs
    dj = d.copy()
    dj.pressure_solver = capi.LINEAR_CG
    c = run(Hydro(dj), u0, q0, 3)
    for sa, sc in zip(a["stats"], c["stats"]):
        assert sa["pressure_residual"] <= 1e-13
        assert sa["pressure_iterations"] * 5 < sc["pressure_iterations"]
    h = Hydro(d)
    h.set_field(capi.F_VELOCITY, u0)
    h.set_field(capi.F_PARTIAL_DENSITY, q0)
    h.init_state()
    for _ in range(3):
        h.step_graph()
    g = {"u": h.get_field(capi.F_VELOCITY), "p": h.get_field(capi.F_PRESSURE),
         "F": h.get_field(capi.F_VOLUME_FLUX), "q": h.get_field(capi.F_PARTIAL_DENSITY)}
    errs = compare(g, a)
    assert all(v <= 1e-12 for v in errs.values()), errs


def test_gauss_seidel_momentum(built):
    """velocity_solver GAUSS_SEIDEL: red-black Gauss-Seidel sweeps in place
    (FP64 rows natural, FP32 rows color-blocked).  Tight solves reach the
    oracle's (lexicographic Gauss-Seidel) fields; fewer sweeps than Jacobi;
    the mixed form within its tolerance; the graph step equals the host
    step."""
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    d, u0, q0, _ = cases.rising_drops(n=24, seed=4, dt_max=5e-3)
    d.n[0], d.n[1], d.n[2] = 24, 20, 16  # nz != nx: the color-blocked index
    from hydro_gb300.cases import cell_centers, two_phase_q
    d.hi[0], d.hi[1], d.hi[2] = 1.5, 1.25, 1.0
    x, y, z = cell_centers(d)
    alpha1 = (((x - 0.7) ** 2 + (y - 0.6) ** 2 + (z - 0.4) ** 2) < 0.2 ** 2).astype(float)
    q0 = two_phase_q(d, alpha1, 2)
    u0 = np.zeros(d.ncells * 3)
    u0[: d.ncells] = 0.05 * np.sin(2 * np.pi * x)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.velocity_solver = capi.LINEAR_GAUSS_SEIDEL
    d.pressure_solver = capi.LINEAR_MGCG
    a = run(Hydro(d), u0, q0, 3)
    do = d.copy()
    do.pressure_solver = capi.LINEAR_CG
    b = run(Oracle(do), u0, q0, 3)
    errs = compare(a, b)
    assert all(v <= 1e-10 for v in errs.values()), errs
    dj = d.copy()
    dj.velocity_solver = capi.LINEAR_JACOBI
    c = run(Hydro(dj), u0, q0, 3)
    assert sum(s["velocity_sweeps"] for s in a["stats"]) < sum(
        s["velocity_sweeps"] for s in c["stats"])
    dm = d.copy()
    dm.precision = capi.MIXED
    dm.velocity_tolerance = 1e-9
    e = run(Hydro(dm), u0, q0, 3)
    errs = compare(e, a)
    assert errs["u"] <= 1e-6 and errs["F"] <= 1e-6 and errs["q"] <= 1e-6, errs
    h = Hydro(dm)
    h.set_field(capi.F_VELOCITY, u0)
    h.set_field(capi.F_PARTIAL_DENSITY, q0)
    h.init_state()
    for _ in range(3):
        h.step_graph()
    g = {"u": h.get_field(capi.F_VELOCITY), "p": h.get_field(capi.F_PRESSURE),
         "F": h.get_field(capi.F_VOLUME_FLUX), "q": h.get_field(capi.F_PARTIAL_DENSITY)}
    errs = compare(g, e)
    assert all(v <= 1e-12 for v in errs.values()), errs


@pytest.mark.parametrize("nx", [25, 24])
def test_gauss_seidel_momentum_2d_cavity(built, nx):
    """Red-black Gauss-Seidel in 2D with rows in cell order (odd nx: FP64
    natural, the mixed form falls back to Jacobi) and color-blocked (even
    nx) against the oracle's lexicographic Gauss-Seidel."""
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    d, u0, q0 = cases.cavity(n=20, mu=0.01, dt=1e-2)
    d.n[0] = nx
    d.hi[0] = nx / 20.0
    u0 = np.zeros(d.ncells * 2)
    q0 = np.ones(d.ncells)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.velocity_solver = capi.LINEAR_GAUSS_SEIDEL
    a = run(Hydro(d), u0, q0, 3)
    b = run(Oracle(d), u0, q0, 3)
    errs = compare(a, b)
    assert all(v <= 1e-10 for v in errs.values()), errs
    dm = d.copy()
    dm.precision = capi.MIXED
    dm.velocity_tolerance = 1e-9
    e = run(Hydro(dm), u0, q0, 3)
    errs = compare(e, a)
    assert errs["u"] <= 1e-6 and errs["F"] <= 1e-6, errs


def test_stencil_solve_matches_oracle(built):
    from hydro_gb300.solver import stencil_solve
    from oracle import oracle as O
    rng = np.random.default_rng(7)
    for dim, n, pin in ((2, (13, 9, 1), -1), (3, (6, 5, 7), 11), (3, (8, 8, 8), -1)):
        nc = n[0] * n[1] * (n[2] if dim == 3 else 1)
        d = capi.default_desc()
        d.dim = dim
        for k in range(3):
            d.n[k] = n[k]
        nf = d.nfaces
        kf = rng.uniform(0.5, 2.0, nf)
        c = rng.normal(size=nc)
        if pin < 0:
            c -= c.mean()
        st, x, it, res = stencil_solve(dim, n, kf, 0.0, pin, 0.3, c, 1e-12, 5000)
        sto, xo, ito, reso = O.stencil_solve(dim, n, kf, 0.0, pin, 0.3, c, 1e-12, 5000)
        assert st == capi.OK and sto == capi.OK
        assert res <= 1e-12
        assert rel(x, xo) <= 1e-9, (dim, n, rel(x, xo))


def test_mass_conservation_and_stats(built):
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    d, u0, q0 = cases.broken_dam(nx=48, ny=24, dt_auto=True, dt_max=5e-4, smooth_times=2)
    d.convergence_tolerance = 1e-6
    d.num_iterations_limit = 30
    h = Hydro(d)
    run(h, u0, q0, 0)
    m0 = h.calc_stat()
    for _ in range(4):
        h.step()
    m1 = h.calc_stat()
    for i in range(2):
        assert abs(m1.partial_mass[i] - m0.partial_mass[i]) <= 1e-11 * abs(m0.partial_mass[i])
    o = Oracle(d)
    run(o, u0, q0, 0)
    so = o.calc_stat()
    for i in range(2):
        assert abs(so.volume[i] - m0.volume[i]) <= 1e-12 * abs(so.volume[i])
        assert abs(so.pd_max[i] - m0.pd_max[i]) <= 1e-12 * abs(so.pd_max[i])


@pytest.mark.parametrize("name", [n for n in __import__("tests.goldens", fromlist=["x"]).names()])
def test_gpu_matches_reference_golden(built, name):
    """GPU against the reference's own outputs (golden vectors)."""
    from hydro_gb300.solver import Hydro
    from tests import goldens
    g = goldens.load(name)
    if not g["gpu_comparable"]:
        pytest.skip("reference LU velocity sweep is a sequential approximate solve")
    d = g["desc"].copy()
    d.velocity_solver = capi.LINEAR_JACOBI
    d.pressure_solver = capi.LINEAR_CG
    d.velocity_tolerance, d.velocity_iters_limit = 1e-14, 20000
    d.pressure_tolerance, d.pressure_iters_limit = 1e-13, 20000
    heat = g["heat"]
    if heat is not None:
        heat = capi.HeatDesc.from_buffer_copy(heat)
        heat.solver, heat.tolerance, heat.iters_limit = capi.LINEAR_JACOBI, 1e-15, 20000
    out = run(Hydro(d), g["u0"], g["q0"], g["nsteps"], heat=heat)
    errs = compare(out, g, capi.fluid_mask(d))
    assert all(v <= 1e-9 for v in errs.values()), errs
    assert [s["outer_iterations"] for s in out["stats"]] == list(g["outer_iterations"])


def test_channel_inlet_outlet_vs_oracle(built):
    """Inlet / outlet (outlet rebalanced every iteration, two phases with
    an inflow of phase 1, split advection): GPU against the oracle, and the
    boundary volume fluxes of CalcStat: inflow of the mixture equals the
    rebalanced outflow."""
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    d, u0, q0 = cases.channel(nx=24, ny=12, dt=1e-2, two_phase=True)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.tvd_split = 1
    a = run(Hydro(d), u0, q0, 3)
    b = run(Oracle(d), u0, q0, 3)
    errs = compare(a, b)
    assert all(v <= 1e-10 for v in errs.values()), errs
    h = Hydro(d)
    run(h, u0, q0, 2)
    o = Oracle(d)
    run(o, u0, q0, 2)
    sg, so = h.calc_stat(), o.calc_stat()
    for i in range(2):
        for k in ("volume_flux_in", "volume_flux_out", "volume"):
            assert getattr(sg, k)[i] == pytest.approx(getattr(so, k)[i], rel=1e-10, abs=1e-14), k
    vin = sg.volume_flux_in[0] + sg.volume_flux_in[1]
    vout = sg.volume_flux_out[0] + sg.volume_flux_out[1]
    assert vin == pytest.approx(1.0, rel=1e-12)   # u_in 1 through a unit-height inlet
    assert vout == pytest.approx(vin, rel=1e-9)


def test_channel_mixed_and_graph(built):
    """The outlet rebalancing inside the mixed path (FP32 mirror of the
    conditions) and inside the graph-captured step."""
    from hydro_gb300.solver import Hydro
    d, u0, q0 = cases.channel(nx=16, ny=8, nz=8, dim=3, dt=1e-2, reverse=True)
    d.pressure_tolerance, d.velocity_tolerance = 1e-10, 1e-12
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    dm = d.copy()
    dm.precision = capi.MIXED
    dm.pressure_solver = capi.LINEAR_MGCG
    ha, hb = Hydro(d), Hydro(dm)
    run(ha, u0, q0, 0)
    run(hb, u0, q0, 0)
    pscale = 0.0
    for _ in range(3):
        ha.step()
        hb.step()
        pa = ha.get_field(capi.F_PRESSURE)
        pscale = max(pscale, float(np.linalg.norm(pa - pa.mean())))
    fields = lambda h: {"u": h.get_field(capi.F_VELOCITY), "p": h.get_field(capi.F_PRESSURE),  # noqa: E731
                        "F": h.get_field(capi.F_VOLUME_FLUX),
                        "q": h.get_field(capi.F_PARTIAL_DENSITY)}
    a, b = fields(ha), fields(hb)
    errs = compare(b, a)
    pa, pb = a["p"] - a["p"].mean(), b["p"] - b["p"].mean()
    p_run = float(np.linalg.norm(pb - pa)) / pscale
    print("mixed vs FP64", errs, "pressure error / largest pressure of the run", p_run)
    # The channel starts from rest: its first step builds a pressure 260x
    # the steady one (rms 87 -> 0.33), and the FP32 rounding of that
    # transient (7e-9 relative) stays in p as an absolute offset, 1.6e-6 of
    # the small steady pressure.  Against the pressure scale of the run it
    # is ~1e-8; velocity and fluxes are within the 1e-6 bar.
    assert errs["u"] <= 1e-6 and errs["F"] <= 1e-6 and errs["q"] <= 1e-6, errs
    assert p_run <= 1e-6, p_run
    assert errs["p"] <= 5e-6, errs
    h = Hydro(dm)
    h.set_field(capi.F_VELOCITY, u0)
    h.set_field(capi.F_PARTIAL_DENSITY, q0)
    h.init_state()
    for _ in range(3):
        h.step_graph()
    c = {"u": h.get_field(capi.F_VELOCITY), "p": h.get_field(capi.F_PRESSURE),
         "F": h.get_field(capi.F_VOLUME_FLUX), "q": h.get_field(capi.F_PARTIAL_DENSITY)}
    errs = compare(c, b)
    assert all(v <= 1e-12 for v in errs.values()), errs


def test_periodic_vs_oracle(built):
    """Periodic directions (x in 2D; x and z in 3D) against the oracle: the
    FP64 path, and the mixed path with the multigrid (periodic coarse
    levels) against the FP64 path."""
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    d, u0, q0 = cases.broken_dam(nx=32, ny=16, dt_auto=False, dt=1e-3, smooth_times=2)
    tight(d)
    d.periodic[0] = 1
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.tvd_split = 1
    a = run(Hydro(d), u0, q0, 3)
    b = run(Oracle(d), u0, q0, 3)
    errs = compare(a, b)
    assert all(v <= 1e-10 for v in errs.values()), errs
    d, u0, q0, _ = cases.rising_drops(n=16, seed=7, dt_max=5e-3)
    d.periodic[0] = d.periodic[2] = 1
    d.gravity[1], d.gravity[2] = -1.0, 0.0  # gravity across the walled direction
    d.pressure_tolerance, d.velocity_tolerance = 1e-10, 1e-12
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    a = run(Hydro(d), u0, q0, 2)
    dm = d.copy()
    dm.precision = capi.MIXED
    dm.pressure_solver = capi.LINEAR_MGCG
    b = run(Hydro(dm), u0, q0, 2)
    errs = compare(b, a)
    assert all(v <= 1e-6 for v in errs.values()), errs
