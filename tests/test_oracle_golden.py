"""The CPU oracle against the reference: golden vectors produced by the
reference's own solver classes (tests/golden/make_golden.py) and the
reference's checked-in sample run of examples/cavity."""
import numpy as np
import pytest

from hydro_gb300 import capi, cases
from tests import goldens
from tests.util import compare, run


@pytest.fixture(scope="module")
def oracle_lib():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.mark.parametrize("name", goldens.names())
def test_oracle_matches_reference(oracle_lib, name):
    g = goldens.load(name)
    o = run(oracle_lib.Oracle(g["desc"]), g["u0"], g["q0"], g["nsteps"], heat=g["heat"])
    errs = compare(o, g, capi.fluid_mask(g["desc"]))
    assert all(v <= 1e-10 for v in errs.values()), errs
    assert [s["outer_iterations"] for s in o["stats"]] == list(g["outer_iterations"])
    assert [s["advection_substeps"] for s in o["stats"]] == list(g["substeps"])
    assert np.allclose([s["dt"] for s in o["stats"]], g["dt"], rtol=1e-12, atol=0)


def test_oracle_reproduces_reference_sample_run(oracle_lib):
    """examples/cavity/sample: 64x64, Re 3200, dt 1e5, 1000 SIMPLE iterations,
    velocity 'lu', pressure Gauss-Seidel with SOR 1.9 and 101 sweeps.  The
    reference printed 6 significant digits."""
    s = goldens.sample()
    d, u0, q0 = cases.cavity(n=64, mu=0.0003125, dt=1e5)
    d.advection_enable = 1
    d.velocity_solver = capi.LINEAR_LU
    d.pressure_solver = capi.LINEAR_GAUSS_SEIDEL
    d.pressure_tolerance, d.pressure_iters_limit, d.pressure_omega = 0.0, 100, 1.9
    d.convergence_tolerance, d.num_iterations_limit = 1e-6, 1000
    o = oracle_lib.Oracle(d, threads=4)
    o.set_field(capi.F_VELOCITY, u0)
    o.set_field(capi.F_PARTIAL_DENSITY, q0)
    o.init_state()
    o.start_step()
    hist = []
    while not o.is_converged():
        o.make_iteration()
        hist.append(o.convergence_indicator())
    o.finish_step()
    ref = s["iter_history"]
    assert len(hist) == len(ref) == 1000
    assert np.max(np.abs(np.array(hist) - ref) / ref) < 1e-5
    u = o.get_field(capi.F_VELOCITY).reshape(2, -1)
    p = o.get_field(capi.F_PRESSURE)
    assert np.max(np.abs(u[0] - s["velocity_x"])) < 1e-6
    assert np.max(np.abs(u[1] - s["velocity_y"])) < 1e-6
    assert np.max(np.abs(p - s["pressure"])) < 1e-6


def test_case_smoothing_matches_oracle(oracle_lib):
    """Initial-field smoothing of the case builders (numpy) equals the
    oracle's GetSmoothField restatement."""
    rng = np.random.default_rng(3)
    for dim, n in ((2, (13, 7, 1)), (3, (5, 6, 4))):
        d = capi.default_desc()
        d.dim = dim
        for k in range(3):
            d.n[k] = n[k]
        a = rng.uniform(size=d.ncells)
        o = oracle_lib.Oracle(d)
        assert np.allclose(cases.smooth(d, a, 3), o.smooth(a, 3), rtol=1e-14, atol=1e-15)


def test_stencil_solve_oracle_residual(oracle_lib):
    rng = np.random.default_rng(1)
    d = capi.default_desc()
    d.dim = 3
    d.n[0], d.n[1], d.n[2] = 7, 6, 5
    kf = rng.uniform(0.5, 1.5, d.nfaces)
    c = rng.normal(size=d.ncells)
    c -= c.mean()
    st, x, it, res = oracle_lib.stencil_solve(3, (7, 6, 5), kf, 0.0, -1, 0.0, c, 1e-12, 2000)
    assert st == capi.OK and res <= 1e-12 and abs(x.mean()) < 1e-12
