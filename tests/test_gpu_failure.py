"""Failure detection through the C-ABI, with every failure made on the host.

The reference checks the pressure for NaN at StartStep and FinishStep and
throws ``std::string`` (fluid.hpp:795-797, 1164-1166), which its module
thread catches (module.cpp:101-107); its linear solvers stop at their
iteration limit and the step goes on (linear.hpp:690-710).  Here:

* a NaN written into an input field with hydro_gpu_set_field makes the
  host-driven and the graph-captured step return HYDRO_ERR_NAN;
* a pressure iteration limit of 1 makes a step complete with
  HYDRO_NOT_CONVERGED (host-driven, graph-captured, and the one case of a
  batch that has the limit), with finite fields and the count of such solves
  in the stats;
* a stencil system with a zero row returns HYDRO_ERR_NAN instead of a
  converged status.

No kernel is made to fault, trap or hang: every loop on the device is bounded
and the statuses are read back on the host.
"""
import numpy as np
import pytest

from hydro_gb300 import capi, cases

pytestmark = pytest.mark.gpu


def _drops(limit=20000, solver=capi.LINEAR_MGCG, precision=capi.MIXED):
    d, u0, q0, _ = cases.rising_drops(n=16, seed=3, dt_max=5e-3)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 2
    d.pressure_solver = solver
    d.precision = precision
    d.pressure_tolerance, d.pressure_iters_limit = 1e-10, limit
    return d, u0, q0


@pytest.mark.parametrize("graph", [False, True])
def test_nan_in_input_field_is_reported(built, graph):
    from hydro_gb300.solver import Hydro, make
    d, u0, q0 = _drops()
    h = make(d, u0, q0)
    st = h.step_graph() if graph else h.step()
    assert st["status"] == capi.OK
    u = h.get_field(capi.F_VELOCITY)
    u[d.ncells // 2] = np.nan
    h.set_field(capi.F_VELOCITY, u)
    with pytest.raises(capi.HydroError) as e:
        h.step_graph() if graph else h.step()
    assert e.value.status == capi.ERR_NAN
    h.close()
    # a fresh context on the same device still works (the failure left the
    # device usable)
    h2 = make(d, u0, q0)
    assert h2.step()["status"] == capi.OK
    assert isinstance(h2, Hydro)


@pytest.mark.parametrize("form", ["fp64_cg", "mixed_mgcg"])
@pytest.mark.parametrize("graph", [False, True])
def test_pressure_limit_gives_not_converged(built, graph, form):
    from hydro_gb300.solver import make
    if form == "fp64_cg":
        d, u0, q0 = _drops(limit=1, solver=capi.LINEAR_CG, precision=capi.FP64)
    else:
        d, u0, q0 = _drops(limit=1)
    h = make(d, u0, q0)
    st = h.step_graph() if graph else h.step()
    assert st["status"] == capi.NOT_CONVERGED, st
    assert st["pressure_unconverged"] >= 1, st
    assert st["pressure_residual"] > d.pressure_tolerance
    for f in (capi.F_VELOCITY, capi.F_PRESSURE, capi.F_VOLUME_FLUX):
        assert np.all(np.isfinite(h.get_field(f)))
    # the same case with its normal limit converges and reports OK
    d.pressure_iters_limit = 20000
    h2 = make(d, u0, q0)
    st2 = h2.step_graph() if graph else h2.step()
    assert st2["status"] == capi.OK and st2["pressure_unconverged"] == 0, st2


def test_batch_reports_the_unconverged_case(built):
    from hydro_gb300.solver import Batch
    d_ok, u0, q0 = _drops()
    d_bad = d_ok.copy()
    d_bad.pressure_iters_limit = 1
    b = Batch([d_ok, d_bad])
    for c in b.cases:
        c.set_field(capi.F_VELOCITY, u0)
        c.set_field(capi.F_PARTIAL_DENSITY, q0)
    b.init_state()
    st = b.step()
    assert st[0]["status"] == capi.OK and st[0]["pressure_unconverged"] == 0
    assert st[1]["status"] == capi.NOT_CONVERGED and st[1]["pressure_unconverged"] >= 1
    b.close()


def test_stencil_zero_row_is_nan_not_converged(built):
    from hydro_gb300.solver import stencil_solve
    n = (8, 6, 1)
    nf = 9 * 6 + 8 * 7
    st, x, it, res = stencil_solve(2, n, np.zeros(nf), 0.0, -1, 0.0,
                                   np.random.default_rng(0).normal(size=48), 1e-10, 100)
    assert st == capi.ERR_NAN
    assert it <= 100
