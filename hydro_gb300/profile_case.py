"""Short, bounded run of the hot path for profiler captures.

    python -m hydro_gb300.profile_case [--n 150] [--precision fp64|mixed]
                                       [--solver cg|mgcg] [--outer 1] [--cg 40]
                                       [--velocity jacobi|gs]

Builds the rising-drops case at n^3, runs one time step with `outer` SIMPLE
iterations and at most `cg` pressure-CG iterations per solve, and exits
(`--solver mgcg`: CG preconditioned by multigrid; `--velocity gs`:
red-black Gauss-Seidel momentum sweeps instead of Jacobi).
At n = 150 the arrays of one CG iteration (p, couplings, diagonal, A p)
exceed the 129 MB L2 while the whole context stays near 2 GB, and the run
issues a few hundred kernel launches -- small enough for ncu captures to end
by themselves.
"""
import argparse
import sys


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=150)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--solver", default="cg", choices=["cg", "mgcg"])
    ap.add_argument("--outer", type=int, default=1)
    ap.add_argument("--cg", type=int, default=40)
    ap.add_argument("--velocity", default="jacobi", choices=["jacobi", "gs"])
    args = ap.parse_args(argv)
    from . import capi, cases
    from .solver import launch_count, make
    d, u0, q0, _ = cases.rising_drops(n=args.n, seed=0, dt_max=2e-3)
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = args.outer
    d.velocity_tolerance = 1e-8
    d.velocity_iters_limit = 50
    if args.velocity == "gs":
        d.velocity_solver = capi.LINEAR_GAUSS_SEIDEL
    d.pressure_tolerance = 1e-30
    d.pressure_iters_limit = args.cg
    d.precision = capi.MIXED if args.precision == "mixed" else capi.FP64
    if args.solver == "mgcg":
        d.pressure_solver = capi.LINEAR_MGCG
    h = make(d, u0, q0)
    st = h.step()
    print("profile_case n=%d %s %s: %s launches=%d"
          % (args.n, args.precision, args.solver, st, launch_count()))
    return 0


if __name__ == "__main__":
    sys.exit(main())
