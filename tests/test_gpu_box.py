"""Rigid box (excluded cells, hydro2d.hpp:306-423) on the GPU: the FP64
path against the oracle on an obstacle in a two-phase channel and on a 3D
box touching a periodic direction; the mixed multigrid path and the
graph-captured step against the FP64 path; the temperature around a box;
the state of the excluded cells left as it was.  (The reference goldens
with a box run in test_gpu_parity.)"""
import numpy as np
import pytest

from hydro_gb300 import capi, cases
from tests.util import compare, rel, run, tight

pytestmark = pytest.mark.gpu


def _box(d, lo, hi):
    d.rigid_box = 1
    for k in range(3):
        d.rigid_box_lo[k], d.rigid_box_hi[k] = lo[k], hi[k]
    return d


def _channel():
    d, u0, q0 = cases.channel(nx=32, ny=16, dt=1e-2, two_phase=True)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.tvd_split = 1
    return _box(d, (0.25, 0.3, 0), (0.45, 0.65, 0)), u0, q0


def _drops():
    d, u0, q0, _ = cases.rising_drops(n=16, seed=5, dt_max=5e-3)
    d.periodic[0] = 1
    d.pressure_tolerance, d.velocity_tolerance = 1e-10, 1e-12
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    return _box(d, (-1.0, 0.2, 0.3), (0.25, 0.45, 0.6)), u0, q0


@pytest.mark.parametrize("make", [_channel, _drops], ids=["channel2d", "drops3d_periodic"])
def test_box_vs_oracle(built, make):
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    d, u0, q0 = make()
    mask = capi.fluid_mask(d)
    assert 0 < (~mask).sum() < mask.size
    a = run(Hydro(d), u0, q0, 3)
    do = d.copy()
    do.pressure_solver = capi.LINEAR_CG
    b = run(Oracle(do), u0, q0, 3)
    errs = compare(a, b, mask)
    assert all(v <= 1e-10 for v in errs.values()), errs
    # excluded cells keep their velocity; no flux through the box
    nc = d.ncells
    u = a["u"].reshape(d.dim, nc)
    u0r = np.asarray(u0).reshape(d.dim, nc)
    assert np.array_equal(u[:, ~mask], u0r[:, ~mask])
    assert np.all(a["p"][~mask] == 0.0)


def test_box_mixed_multigrid_and_graph(built):
    from hydro_gb300.solver import Hydro
    d, u0, q0 = _drops()
    d.periodic[0] = 0
    mask = capi.fluid_mask(d)
    a = run(Hydro(d), u0, q0, 3)
    dm = d.copy()
    dm.precision = capi.MIXED
    dm.pressure_solver = capi.LINEAR_MGCG
    b = run(Hydro(dm), u0, q0, 3)
    errs = compare(b, a, mask)
    print("mixed vs FP64", errs)
    # measured: u 1.2e-7, p 2.3e-9
    assert all(v <= 1e-6 for v in errs.values()), errs
    h = Hydro(dm)
    h.set_field(capi.F_VELOCITY, u0)
    h.set_field(capi.F_PARTIAL_DENSITY, q0)
    h.init_state()
    for _ in range(3):
        h.step_graph()
    c = {"u": h.get_field(capi.F_VELOCITY), "p": h.get_field(capi.F_PRESSURE),
         "F": h.get_field(capi.F_VOLUME_FLUX), "q": h.get_field(capi.F_PARTIAL_DENSITY)}
    errs = compare(c, b, mask)
    assert all(v <= 1e-12 for v in errs.values()), errs


def test_box_heat_vs_oracle(built):
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    d, u0, q0 = _channel()
    h = capi.default_heat_desc(d.dt)
    h.temperature_initial = 0.25
    h.conductivity[0], h.conductivity[1] = 0.6, 0.025
    # the box over the inlet and the obstacle's upstream face
    for k, (lo, hi) in enumerate(((-1.0, 0.3), (-1.0, 2.0), (-1.0, 1.0))):
        h.box_lo[k], h.box_hi[k] = lo, hi
    h.box_temperature = 1.0
    h.tolerance, h.iters_limit = 1e-15, 20000
    a = run(Hydro(d), u0, q0, 3, heat=h)
    ho = capi.HeatDesc.from_buffer_copy(h)
    ho.solver = capi.LINEAR_GAUSS_SEIDEL
    do = d.copy()
    do.pressure_solver = capi.LINEAR_CG
    b = run(Oracle(do), u0, q0, 3, heat=ho)
    assert rel(a["T"], b["T"]) <= 1e-10
    mask = capi.fluid_mask(d)
    assert np.all(a["T"][~mask] == 0.25)  # identity rows inside the box


def test_box_rejections(built):
    from hydro_gb300.solver import Hydro
    d, u0, q0 = _channel()
    d.simpler = 1
    with pytest.raises(capi.HydroError):
        Hydro(d)
    d, u0, q0 = _channel()
    mask = capi.fluid_mask(d)
    d.pressure_fixed_cell = int(np.flatnonzero(~mask)[0])
    with pytest.raises(capi.HydroError):
        Hydro(d)
