"""Generates the golden vectors of the parity tests from the reference.

Run in a container that holds the reference tree (default /root/reference;
override with HYDRO_REFERENCE):

    make -C oracle            # builds oracle/_ref/libhydro_ref.so from it
    python tests/golden/make_golden.py [case ...]   # all, or the named cases

1. For each case below, the reference's own FluidSimple +
   AdvectionSolverMultiExplicit (driven by oracle/ref_harness.cpp) runs
   from the stated initial fields; inputs, final fields and per-step
   statistics go to tests/golden/<name>.npz.
2. The reference's checked-in sample run of examples/cavity (64x64,
   Re 3200, 1000 SIMPLE iterations) is read from its .vts / .plt output and
   stored as tests/golden/cavity_sample.npz (6 significant digits, as
   printed by the reference).
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hydro_gb300 import capi, cases  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF = os.environ.get("HYDRO_REFERENCE", "/root/reference")


def tight(d, solver=capi.LINEAR_GAUSS_SEIDEL, p_tol=1e-14):
    """Linear solves to rounding level: the reference's Gauss-Seidel stops
    on max |update| (linear.hpp:710), so its tolerance is absolute and is set
    near the rounding level of the case's pressure scale."""
    d.velocity_solver = solver
    d.pressure_solver = capi.LINEAR_GAUSS_SEIDEL
    d.velocity_tolerance = 1e-14
    d.velocity_iters_limit = 1000000
    d.pressure_tolerance = p_tol
    d.pressure_iters_limit = 1000000
    d.pressure_omega = 1.5
    return d


def heat(dt, lo, hi, second_order=1, relax=1.0):
    """Temperature of the heat goldens: 0.25 initially, the given box at 1,
    conductivities 0.6 / 0.025, Gauss-Seidel to 1e-15 (tight)."""
    h = capi.default_heat_desc(dt)
    h.temperature_initial = 0.25
    h.conductivity[0], h.conductivity[1] = 0.6, 0.025
    for k in range(3):
        h.box_lo[k], h.box_hi[k] = lo[k], hi[k]
    h.box_temperature = 1.0
    h.time_second_order = second_order
    h.relaxation_factor = relax
    h.solver = capi.LINEAR_GAUSS_SEIDEL
    h.tolerance, h.iters_limit = 1e-15, 1000000
    return h


def golden_cases():
    out = []
    d, u0, q0 = cases.cavity(n=16, mu=0.01, dt=1e-2)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    out.append(("cavity2d_fixed", d, u0, q0, 3, True))

    d, u0, q0 = cases.cavity(n=16, mu=0.01, dt=1e-2)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 1e-9, 200
    out.append(("cavity2d_converged", d, u0, q0, 2, True))

    d, u0, q0 = cases.broken_dam(nx=40, ny=20, dt_auto=True, dt_max=5e-4, smooth_times=2)
    tight(d, p_tol=1e-10)
    d.convergence_tolerance, d.num_iterations_limit = 1e-7, 40
    out.append(("dam2d_auto", d, u0, q0, 3, True))

    d, u0, q0 = cases.broken_dam(nx=24, ny=12, dt_auto=False, dt=1e-3, smooth_times=1)
    tight(d, p_tol=1e-10)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 2
    d.tvd_split, d.sigma, d.force_geometric_average = 1, 0.05, 1
    out.append(("dam2d_split_sigma_geo", d, u0, q0, 2, True))

    d, u0, q0, _ = cases.rising_drops(n=12, seed=3, dt_max=5e-3)
    tight(d, p_tol=1e-12)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    out.append(("drops3d", d, u0, q0, 2, True))

    d, u0, q0 = cases.cavity(n=10, dim=3, dt=1e-2)
    d.n[2] = 7
    u0, q0 = np.zeros(d.ncells * 3), np.ones(d.ncells)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.pressure_fixed_cell, d.time_second_order = 123, 0
    out.append(("cavity3d_pinned_first_order", d, u0, q0, 2, True))

    d, u0, q0 = cases.cavity(n=12, mu=0.02, dt=5e-3)
    d.n[0], d.n[1], d.hi[0] = 20, 12, 1.7
    u0, q0 = np.zeros(d.ncells * 2), np.ones(d.ncells)
    tight(d, capi.LINEAR_JACOBI)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 4
    d.guess_extrapolation, d.velocity_relaxation_factor = 0.5, 0.7
    out.append(("cavity2d_jacobi_extrap", d, u0, q0, 3, True))

    # inlet / outlet (UpdateOutletBaseConditions, fluid.hpp:542-600)
    d, u0, q0 = cases.channel(nx=24, ny=10, dt=1e-2)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    out.append(("channel2d", d, u0, q0, 3, True))

    d, u0, q0 = cases.channel(nx=20, ny=8, dt=1e-2, reverse=True, two_phase=True)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.tvd_split = 1
    out.append(("channel2d_reverse_two_phase", d, u0, q0, 3, True))

    d, u0, q0 = cases.channel(nx=10, ny=6, nz=5, dim=3, dt=1e-2)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 2
    d.pressure_fixed_cell = 7
    out.append(("channel3d_pinned", d, u0, q0, 2, True))

    # periodicity (mesh2d.hpp / mesh3d.hpp PERX, PERZ): a two-phase layer
    # periodic in x; a 3D box periodic in x and z with a moving lid
    d, u0, q0 = cases.broken_dam(nx=24, ny=12, dt_auto=False, dt=1e-3, smooth_times=2)
    tight(d, p_tol=1e-10)
    d.periodic[0] = 1
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.tvd_split = 1
    out.append(("dam2d_periodic_x", d, u0, q0, 2, True))

    d, u0, q0 = cases.cavity(n=8, dim=3, dt=1e-2)
    d.n[0], d.n[2] = 10, 6
    u0, q0 = np.zeros(d.ncells * 3), np.ones(d.ncells)
    u0[: d.ncells] = 0.1 * np.sin(2 * np.pi * (np.arange(d.ncells) % 10) / 10.0)
    tight(d)
    d.periodic[0] = d.periodic[2] = 1
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    out.append(("box3d_periodic_xz", d, u0, q0, 2, True))

    # SIMPLER (fluid.hpp:1059-1155): singular walls, pinned two-phase
    d, u0, q0 = cases.cavity(n=16, mu=0.01, dt=1e-2)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.simpler = 1
    out.append(("cavity2d_simpler", d, u0, q0, 3, True))

    d, u0, q0 = cases.broken_dam(nx=24, ny=12, dt_auto=False, dt=1e-3, smooth_times=2)
    tight(d, p_tol=1e-10)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.simpler = 1
    d.pressure_fixed_cell = 30
    out.append(("dam2d_simpler_pinned", d, u0, q0, 2, True))

    # HeatSolver attached (hydro2d.hpp:650-687): the temperature is the
    # eighth element of the case tuple
    d, u0, q0 = cases.broken_dam(nx=24, ny=12, dt_auto=False, dt=1e-3, smooth_times=2)
    tight(d, p_tol=1e-10)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    h = heat(d.dt, lo=(-1.0, -1.0, -1.0), hi=(0.3, 0.02, 10.0))
    out.append(("heat_dam2d", d, u0, q0, 3, True, h))

    d, u0, q0 = cases.channel(nx=12, ny=6, nz=4, dim=3, dt=1e-2, two_phase=True)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 2
    # box over the inlet side (x = 0, lower half in y): inflow carries T = 1
    h = heat(d.dt, lo=(-1.0, -1.0, -1.0), hi=(0.0, 0.5, 10.0), second_order=0, relax=0.9)
    h.conductivity[1] = 0.2
    out.append(("heat_channel3d", d, u0, q0, 3, True, h))

    d, u0, q0 = cases.broken_dam(nx=16, ny=8, dt_auto=False, dt=1e-3, smooth_times=2)
    tight(d, p_tol=1e-10)
    d.periodic[0] = 1
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 2
    h = heat(d.dt, lo=(0.25, -1.0, -1.0), hi=(0.6, 0.0, 10.0))
    out.append(("heat_dam2d_periodic_x", d, u0, q0, 2, True, h))

    # rigid box (hydro2d.hpp:306-423): excluded cells, walls at rest
    # around them; in a channel (obstacle in the stream), touching the
    # bottom wall of a cavity, on the floor under a breaking dam, in 3D
    def box(d, lo, hi):
        d.rigid_box = 1
        for k in range(3):
            d.rigid_box_lo[k], d.rigid_box_hi[k] = lo[k], hi[k]
        return d

    d, u0, q0 = cases.channel(nx=24, ny=12, dt=1e-2, two_phase=True)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    out.append(("box_channel2d", box(d, (0.3, 0.3, 0), (0.5, 0.6, 0)), u0, q0, 3, True))

    d, u0, q0 = cases.cavity(n=16, mu=0.01, dt=1e-2)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    out.append(("box_cavity2d", box(d, (0.3, 0.0, 0), (0.55, 0.4, 0)), u0, q0, 3, True))

    d, u0, q0 = cases.broken_dam(nx=24, ny=12, dt_auto=False, dt=1e-3, smooth_times=2)
    tight(d, p_tol=1e-10)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    out.append(("box_dam2d", box(d, (1.8, -1.0, 0), (2.4, 0.45, 0)), u0, q0, 2, True))

    d, u0, q0 = cases.cavity(n=8, dim=3, dt=1e-2)
    d.n[0], d.n[2] = 10, 6
    u0, q0 = np.zeros(d.ncells * 3), np.ones(d.ncells)
    u0[: d.ncells] = 0.1 * np.sin(2 * np.pi * (np.arange(d.ncells) % 10) / 10.0)
    tight(d)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    out.append(("box_cavity3d", box(d, (0.3, 0.2, 0.3), (0.65, 0.6, 0.7)), u0, q0, 2, True))

    # a box across the periodic end of x (harness built with PERX)
    d, u0, q0, _ = cases.rising_drops(n=12, seed=5, dt_max=5e-3)
    d.periodic[0] = 1
    tight(d, p_tol=1e-12)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 2
    out.append(("box_drops3d_periodic_x", box(d, (-1.0, 0.2, 0.3), (0.25, 0.45, 0.6)), u0, q0, 2,
                True))

    # reference defaults for the linear solvers: one LU sweep for velocity
    # (an approximate solve; CPU-only semantics), SOR pressure
    d, u0, q0 = cases.broken_dam(nx=16, ny=8, dt_auto=False, dt=2e-3, smooth_times=2)
    d.velocity_solver = capi.LINEAR_LU
    d.pressure_solver = capi.LINEAR_GAUSS_SEIDEL
    d.pressure_tolerance, d.pressure_iters_limit, d.pressure_omega = 1e-3, 1000, 1.9
    d.convergence_tolerance, d.num_iterations_limit = 1e-2, 10
    d.sharp = 0.5
    out.append(("dam2d_lu_sor_sharp", d, u0, q0, 3, False))

    # interface sharpening (advection.hpp:481-530) with tight linear solves
    # (Jacobi velocity sweeps), which the GPU path reproduces
    d, u0, q0 = cases.broken_dam(nx=24, ny=12, dt_auto=False, dt=2e-3, smooth_times=2)
    tight(d, solver=capi.LINEAR_JACOBI, p_tol=1e-10)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 3
    d.sharp = 0.5
    out.append(("dam2d_sharp", d, u0, q0, 3, True))
    return out


def make_cases(only=None):
    for case in golden_cases():
        name, d, u0, q0, nsteps, gpu_ok = case[:6]
        if only and name not in only:
            continue
        extra = {}
        if len(case) > 6:
            u, p, F, q, T, stats = O.ref_run_heat(d, case[6], u0, q0, nsteps)
            extra = {"heat": json.dumps(capi.heat_to_dict(case[6])), "T": T}
        else:
            u, p, F, q, stats = O.ref_run(d, u0, q0, nsteps)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(
            path, desc=json.dumps(capi.desc_to_dict(d)), u0=u0, q0=q0, nsteps=nsteps,
            gpu_comparable=gpu_ok, u=u, p=p, F=F, q=q, **extra,
            outer_iterations=np.array([s["outer_iterations"] for s in stats]),
            indicator=np.array([s["convergence_indicator"] for s in stats]),
            dt=np.array([s["dt"] for s in stats]),
            substeps=np.array([s["advection_substeps"] for s in stats]))
        print("wrote", path, [s["outer_iterations"] for s in stats])


def make_sample():
    sdir = os.path.join(REF, "examples", "cavity", "sample")
    vts = open(os.path.join(sdir, "exp.field.0.vts")).read()

    def arr(name):
        m = re.search(r'Name="%s"[^>]*>\s*([^<]*)<' % name, vts)
        return np.array([float(v) for v in m.group(1).split()])

    hist = []
    for line in open(os.path.join(sdir, "exp.iter_history.plt")):
        if re.match(r"^\d+ ", line):
            hist.append(float(line.split()[1]))
    path = os.path.join(HERE, "cavity_sample.npz")
    np.savez_compressed(path, velocity_x=arr("velocity_x"), velocity_y=arr("velocity_y"),
                        pressure=arr("pressure"), iter_history=np.array(hist))
    print("wrote", path)


def make_vts():
    """Frames of the reference's ParaView writer for seeded fields on small
    2D and 3D blocks (values of mixed sign and magnitude), with the entry
    set the defaults select; the inputs are stored beside the output."""
    import tempfile
    rng = np.random.default_rng(20261203)
    for name, dim, n, lo, hi in (("vts2d", 2, (5, 3, 1), (0.0, -0.5, 0.0), (1.25, 0.7, 1.0)),
                                 ("vts3d", 3, (3, 2, 4), (0.0, 0.0, 0.0), (1.0, 0.5, 2.0))):
        nc = n[0] * n[1] * n[2]
        nnode = (n[0] + 1) * (n[1] + 1) * ((n[2] + 1) if dim == 3 else 1)
        hx = [(hi[k] - lo[k]) for k in range(3)]
        nodes = {}
        idx = np.arange(nnode)
        ii = idx % (n[0] + 1)
        jj = (idx // (n[0] + 1)) % (n[1] + 1)
        kk = idx // ((n[0] + 1) * (n[1] + 1))
        nodes["x"] = lo[0] + (ii / n[0]) * hx[0]
        nodes["y"] = lo[1] + (jj / n[1]) * hx[1]
        if dim == 3:
            nodes["z"] = lo[2] + (kk / n[2]) * hx[2]
        cells = {"velocity_x": rng.normal(size=nc) * 1e-3,
                 "velocity_y": rng.normal(size=nc) * 10.0 ** rng.integers(-6, 3, size=nc)}
        if dim == 3:
            cells["velocity_z"] = rng.normal(size=nc)
        cells["pressure"] = rng.uniform(-1, 1, size=nc) * 1234.5678
        cells["volume_fraction_0"] = np.clip(rng.uniform(-0.2, 1.2, size=nc), 0, 1)
        cells["volume_fraction_1"] = 1.0 - cells["volume_fraction_0"]
        times = [0.0, 0.0125]
        with tempfile.TemporaryDirectory() as td:
            cwd = os.getcwd()
            os.chdir(td)
            try:
                O.ref_write_vts(dim, n, lo, hi, nodes, cells, name + ".field", times)
                frames = [open(name + ".field.%d.vts" % k).read() for k in range(len(times))]
                pvd = open(name + ".field.pvd").read()
            finally:
                os.chdir(cwd)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, dim=dim, n=np.array(n), lo=np.array(lo), hi=np.array(hi),
                            node_names=np.array(list(nodes)), cell_names=np.array(list(cells)),
                            times=np.array(times), frames=np.array(frames), pvd=pvd,
                            **{"node_" + k: v for k, v in nodes.items()},
                            **{"cell_" + k: v for k, v in cells.items()})
        print("wrote", path)


if __name__ == "__main__":
    if not O.ref_available():
        O.build(ref=True)
    # optional: names of solver cases to (re)write, e.g. dam2d_sharp
    only = set(sys.argv[1:])
    make_cases(only)
    if not only:
        make_vts()
        make_sample()
