"""Speed of the CPU port (liboracle.so, the plain-C restatement timed as the
benchmark's CPU baseline) against the reference's own solver classes
(oracle/_ref/libhydro_ref_omp.so: the reference headers compiled unchanged
with -O3 -fopenmp), on the same case and the reference's default linear
solvers: one LU sweep for velocity, SOR (omega 1.9) to a max update of 1e-3,
at most 1000 sweeps, for pressure.  Runs where the reference tree is present
(the _ref build needs it); prints seconds per step of both and the ratio.

    python oracle/time_port.py [--n 64] [--steps 2] [--threads N]
"""
import argparse
import ctypes
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
# the repository root, not this folder, names the `oracle` package
sys.path[0] = os.path.dirname(HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args()
    import subprocess
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so", "ref-omp"], check=True)
    lib_ref = os.path.join(HERE, "_ref", "libhydro_ref_omp.so")
    if not os.path.exists(lib_ref):
        print("reference harness not built (no reference tree): nothing to compare")
        return 0
    os.environ["OMP_NUM_THREADS"] = str(a.threads)
    from hydro_gb300 import capi, cases
    from oracle import oracle as O
    d, u0, q0, _ = cases.rising_drops(n=a.n, seed=a.seed, dt_max=2e-3)
    d.convergence_tolerance, d.num_iterations_limit = 0.0, 5
    d.velocity_solver = capi.LINEAR_LU
    d.pressure_solver = capi.LINEAR_GAUSS_SEIDEL
    d.pressure_omega, d.pressure_tolerance, d.pressure_iters_limit = 1.9, 1e-3, 1000
    R = ctypes.CDLL(lib_ref)
    D = ctypes.POINTER(ctypes.c_double)
    R.ref_run.argtypes = [ctypes.POINTER(capi.HydroDesc), D, D, ctypes.c_int, D, D, D, D,
                          ctypes.POINTER(capi.StepStats)]
    R.ref_run.restype = ctypes.c_int
    import numpy as np
    nc, nf = d.ncells, d.nfaces
    outs = [np.empty(nc * 3), np.empty(nc), np.empty(nf), np.empty(nc * 2)]
    stats = (capi.StepStats * a.steps)()
    dd = d.copy()
    t0 = time.perf_counter()
    st = R.ref_run(ctypes.byref(dd), O._dp(np.ascontiguousarray(u0)),
                   O._dp(np.ascontiguousarray(q0)), a.steps, *[O._dp(o) for o in outs], stats)
    t_ref = time.perf_counter() - t0
    assert st == 0, st
    sweeps_ref = [stats[i].pressure_iterations for i in range(a.steps)]
    o = O.Oracle(d, threads=a.threads)
    o.set_field(capi.F_VELOCITY, u0)
    o.set_field(capi.F_PARTIAL_DENSITY, q0)
    o.init_state()
    t0 = time.perf_counter()
    st_port = [o.step() for _ in range(a.steps)]
    t_port = time.perf_counter() - t0
    sweeps_port = [s["pressure_iterations"] for s in st_port]
    print("rising drops %d^3, %d steps from rest, %d threads" % (a.n, a.steps, a.threads))
    print("reference (headers, -O3 -fopenmp): %.2f s/step, SOR sweeps per step %s"
          % (t_ref / a.steps, sweeps_ref))
    print("port (liboracle.so, -O2 -fopenmp):  %.2f s/step, SOR sweeps per step %s"
          % (t_port / a.steps, sweeps_port))
    print("port / reference time: %.2f" % (t_port / t_ref))
    return 0


if __name__ == "__main__":
    sys.exit(main())
