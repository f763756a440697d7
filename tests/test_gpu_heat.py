"""Temperature (HeatSolver, heat.hpp:18-94) on the GPU: against the oracle
on cases the reference goldens do not cover (2D channel with the box over
the inlet, 3D rising drops with a box on the floor, a periodic direction),
the graph-captured and batched steps against the host-driven step, the
mixed-precision fluid with FP64 temperature, and the temperature entry of
the field writer."""
import re

import numpy as np
import pytest

from hydro_gb300 import capi, cases
from tests.util import compare, rel, run, tight

pytestmark = pytest.mark.gpu


def _heat(dt, lo, hi, second_order=1, relax=1.0):
    h = capi.default_heat_desc(dt)
    h.temperature_initial = 0.25
    h.conductivity[0], h.conductivity[1] = 0.6, 0.025
    for k in range(3):
        h.box_lo[k], h.box_hi[k] = lo[k], hi[k]
    h.box_temperature = 1.0
    h.time_second_order = second_order
    h.relaxation_factor = relax
    h.tolerance, h.iters_limit = 1e-15, 20000
    return h


def _cases():
    out = []
    d, u0, q0 = cases.channel(nx=24, ny=12, dt=1e-2, two_phase=True)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    out.append(("channel2d", d, u0, q0, _heat(d.dt, (-1, -1, -1), (0.0, 0.5, 9)), 3))
    d, u0, q0, _ = cases.rising_drops(n=16, seed=3, dt_max=5e-3)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 2
    out.append(("drops3d", d, u0, q0,
                _heat(5e-3, (-1, -1, -1), (0.5, 0.0, 9), second_order=0, relax=0.8), 2))
    d, u0, q0 = cases.broken_dam(nx=32, ny=16, dt_auto=False, dt=1e-3, smooth_times=2)
    tight(d)
    d.periodic[0] = 1
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 2
    out.append(("dam2d_periodic", d, u0, q0, _heat(d.dt, (0.3, -1, -1), (0.7, 0.0, 9)), 3))
    return out


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
def test_heat_vs_oracle(built, case):
    from hydro_gb300.solver import Hydro
    from oracle.oracle import Oracle
    _, d, u0, q0, h, nsteps = case
    a = run(Hydro(d), u0, q0, nsteps, heat=h)
    ho = capi.HeatDesc.from_buffer_copy(h)
    ho.solver = capi.LINEAR_GAUSS_SEIDEL
    b = run(Oracle(d), u0, q0, nsteps, heat=ho)
    errs = compare(a, b)
    assert all(v <= 1e-10 for v in errs.values()), errs
    assert np.ptp(b["T"]) > 1e-3  # the temperature moved


def test_heat_graph_and_batch_match_host_step(built):
    from hydro_gb300.solver import Batch, Hydro
    _, d, u0, q0, h, nsteps = _cases()[0]
    ref = run(Hydro(d), u0, q0, nsteps, heat=h)
    g = Hydro(d)
    g.set_field(capi.F_VELOCITY, u0)
    g.set_field(capi.F_PARTIAL_DENSITY, q0)
    g.init_state()
    g.heat_create(h)
    for _ in range(nsteps):
        g.step_graph()
    assert rel(g.temperature(), ref["T"]) <= 1e-13
    tp = g.temperature(capi.TIME_PREV)
    assert np.all(np.isfinite(tp)) and rel(tp, ref["T"]) > 0  # the previous layer
    _, d2, u2, q2, h2, _ = _cases()[2]
    b = Batch([d, d2])
    for c, (uu, qq) in zip(b.cases, ((u0, q0), (u2, q2))):
        c.set_field(capi.F_VELOCITY, uu)
        c.set_field(capi.F_PARTIAL_DENSITY, qq)
    b.init_state()
    b.cases[0].heat_create(h)
    b.cases[1].heat_create(h2)
    for _ in range(nsteps):
        b.step()
    ref2 = run(Hydro(d2), u2, q2, nsteps, heat=h2)
    assert rel(b.cases[0].temperature(), ref["T"]) <= 1e-13
    assert rel(b.cases[1].temperature(), ref2["T"]) <= 1e-13


def test_heat_with_mixed_fluid(built):
    """The temperature stays FP64 when the fluid runs the mixed path; its
    error follows the fluid's (volume fluxes within 1e-6)."""
    from hydro_gb300.solver import Hydro
    _, d, u0, q0, h, nsteps = _cases()[1]
    d.pressure_tolerance, d.velocity_tolerance = 1e-10, 1e-12
    a = run(Hydro(d), u0, q0, nsteps, heat=h)
    dm = d.copy()
    dm.precision = capi.MIXED
    dm.pressure_solver = capi.LINEAR_MGCG
    b = run(Hydro(dm), u0, q0, nsteps, heat=h)
    assert rel(b["F"], a["F"]) <= 1e-6
    assert rel(b["T"], a["T"]) <= 1e-6


def test_heat_rejects_bad_desc_and_output_entry(built, tmp_path):
    from hydro_gb300.solver import Hydro
    _, d, u0, q0, h, _ = _cases()[0]
    x = Hydro(d)
    x.set_field(capi.F_VELOCITY, u0)
    x.set_field(capi.F_PARTIAL_DENSITY, q0)
    x.init_state()
    with pytest.raises(capi.HydroError):
        x.temperature()  # no heat attached
    lib = capi.load()
    outp = capi.ctypes.c_void_p()
    base = str(tmp_path / "t").encode()
    assert lib.hydro_output_open(x.ctx, base, b"temperature", capi.ctypes.byref(outp)) == capi.ERR_ARG
    bad = capi.HeatDesc.from_buffer_copy(h)
    bad.dt = 0.0
    with pytest.raises(capi.HydroError):
        x.heat_create(bad)
    x.heat_create(h)
    x.step()
    assert lib.hydro_output_open(x.ctx, base, b"x,y,temperature",
                                 capi.ctypes.byref(outp)) == capi.OK
    assert lib.hydro_output_write(outp, capi.ctypes.c_double(0.5)) == capi.OK
    assert lib.hydro_output_close(outp) == capi.OK
    text = open(str(tmp_path / "t.0.vts")).read()
    m = re.search(r'Name="temperature"[^>]*>\s*([^<]*)<', text)
    vals = np.array([float(v) for v in m.group(1).split()])
    assert np.allclose(vals, x.temperature(), rtol=1e-5, atol=0)
