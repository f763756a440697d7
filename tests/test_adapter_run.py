"""The reference-side adapter run, not only compiled: the reference's own
harness (oracle/ref_harness.cpp) built with FluidSimpleGpu and
AdvectionSolverMultiGpu (hydro_gb300/adapter/fluid_simple_gpu.hpp) in place
of FluidSimple and AdvectionSolverMultiExplicit -- the same constructor
arguments, the same StartStep / MakeIteration / FinishStep /
GetVelocity / GetField calls of the FluidSolver and AdvectionSolverMulti
interfaces -- must reproduce the reference's golden fields.

The adapter needs the reference's headers to compile, which exist only in
this container, and a GPU to run the library behind its C-ABI, which
exists only on the GPU machine; so here the C-ABI is forwarded to the CPU
oracle (oracle/adapter_shim.c).  What this pins is the adapter: the
translation of the reference's conditions, rigid box and pinned cell into
the description, the component-major / raw-order field marshalling, the
layer indices, the time-step and sub-step sequence.  The library behind the
same entry points is pinned against the oracle and the same goldens by the
GPU tests.  Skipped where the reference tree is absent."""
import numpy as np
import pytest

from hydro_gb300 import capi
from oracle import oracle as O
from tests import goldens
from tests.util import compare

REF_LIB = O.REF_LIB.replace(".so", "_adapter.so")


def _cases():
    out = []
    for name in goldens.names():
        g = goldens.load(name)
        d = g["desc"]
        if not g["gpu_comparable"] or g["heat"] is not None or any(d.periodic[:d.dim]):
            continue
        out.append(name)
    return out


@pytest.fixture(scope="module")
def adapter_lib():
    import os
    import subprocess
    subprocess.run(["make", "-s", "-C", O.HERE, "adapter"], check=True)
    if not os.path.exists(REF_LIB):
        pytest.skip("reference tree not present: the adapter cannot be compiled")
    return O.ref_lib("adapter")


@pytest.mark.parametrize("name", _cases())
def test_adapter_reproduces_reference_golden(adapter_lib, name):
    g = goldens.load(name)
    d = g["desc"].copy()
    # the adapter's solves: Jacobi velocity sweeps and CG pressure, tight
    d.velocity_tolerance, d.velocity_iters_limit = 1e-14, 20000
    d.pressure_tolerance, d.pressure_iters_limit = 1e-13, 20000
    u, p, F, q, stats = O.ref_run(d, g["u0"], g["q0"], g["nsteps"], variant="adapter")
    errs = compare({"u": u, "p": p, "F": F, "q": q}, g, capi.fluid_mask(d))
    assert all(v <= 1e-9 for v in errs.values()), errs
    assert [s["outer_iterations"] for s in stats] == list(g["outer_iterations"])
    assert np.allclose([s["dt"] for s in stats], g["dt"], rtol=1e-12, atol=0)


def test_adapter_nan_throws_the_reference_string(adapter_lib):
    """A NaN reaching the pressure makes the adapter throw std::string, as
    FluidSimple does (fluid.hpp:795-797, 1164-1166); the harness catches it
    like the module thread (module.cpp:101-107) and reports HYDRO_ERR_NAN."""
    g = goldens.load("cavity2d_fixed")
    u0 = np.array(g["u0"], dtype=np.float64)
    u0[len(u0) // 3] = np.nan
    with pytest.raises(capi.HydroError) as e:
        O.ref_run(g["desc"], u0, g["q0"], 2, variant="adapter")
    assert e.value.status == capi.ERR_NAN
