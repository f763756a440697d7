"""The reference-side C++ adapter (hydro_gb300/adapter/fluid_simple_gpu.hpp)
compiles against the reference's own headers, 2D and 3D, with every member
instantiated.  Needs the reference tree (HYDRO_REFERENCE, default
/root/reference); skipped where it is absent."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("HYDRO_REFERENCE", "/root/reference")

SRC = r'''
#include "mesh2d.hpp"
#include "mesh3d.hpp"
#include "fluid.hpp"
#include "advection.hpp"
#include "conv_diff.hpp"
#include "fluid_simple_gpu.hpp"
template class solver::FluidSimpleGpu<geom::geom2d::MeshStructured<double>>;
template class solver::FluidSimpleGpu<geom::geom3d::MeshStructured<double>>;
template class solver::AdvectionSolverMultiGpu<geom::geom2d::MeshStructured<double>>;
template class solver::AdvectionSolverMultiGpu<geom::geom3d::MeshStructured<double>>;
template class solver::HeatSolverGpu<geom::geom2d::MeshStructured<double>>;
template class solver::HeatSolverGpu<geom::geom3d::MeshStructured<double>>;
int main() { return 0; }
'''


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "source", "hydro2dmpi")),
                    reason="reference tree not present")
def test_adapter_compiles_against_reference(tmp_path):
    src = tmp_path / "adapter_tu.cpp"
    src.write_text(SRC)
    cmd = ["g++", "-std=c++11", "-fsyntax-only", "-w",
           "-I", os.path.join(REF, "source", "hydro2dmpi"),
           "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "hydro_gb300", "adapter"), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
