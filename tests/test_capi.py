"""The C-ABI library without a GPU: it loads, exports every entry point
include/hydro_gpu.h declares, its structures have the layout the header
gives, defaults match examples/general.hydroconf, and creating a context
without a device fails loudly (no CPU fallback)."""
import ctypes
import os
import re
import subprocess

import pytest

from hydro_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hydro_gpu.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hydro_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib(built):
    return capi.load()


def test_exports_every_declared_symbol(lib):
    names = declared()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", capi.lib_path()], capture_output=True,
                         text=True, check=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if " T " in l)
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    fields = [f for f, _ in capi.HydroDesc._fields_]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "hydro_gpu.h"',
             "int main(void) {",
             '  printf("%zu %zu %zu\\n", sizeof(hydro_desc), sizeof(hydro_step_stats), sizeof(hydro_stat));']
    for f in fields:
        lines.append('  printf("%%zu\\n", offsetof(hydro_desc, %s));' % f)
    hfields = [f for f, _ in capi.HeatDesc._fields_]
    lines.append('  printf("%zu\\n", sizeof(hydro_heat_desc));')
    for f in hfields:
        lines.append('  printf("%%zu\\n", offsetof(hydro_heat_desc, %s));' % f)
    lines.append("  return 0; }")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == ctypes.sizeof(capi.HydroDesc)
    assert int(out[1]) == ctypes.sizeof(capi.StepStats)
    assert int(out[2]) == ctypes.sizeof(capi.Stat)
    for f, off in zip(fields, out[3:3 + len(fields)]):
        assert getattr(capi.HydroDesc, f).offset == int(off), f
    rest = out[3 + len(fields):]
    assert int(rest[0]) == ctypes.sizeof(capi.HeatDesc)
    for f, off in zip(hfields, rest[1:]):
        assert getattr(capi.HeatDesc, f).offset == int(off), f


def test_desc_default_matches_python(lib):
    d = capi.HydroDesc()
    assert lib.hydro_desc_default(ctypes.byref(d)) == capi.OK
    assert capi.desc_to_dict(d) == capi.desc_to_dict(capi.default_desc())


def test_create_rejects_bad_desc(lib):
    d = capi.default_desc()
    ctx = ctypes.c_void_p()
    d.simpler = 1
    d.precision = capi.MIXED  # SIMPLER runs on the FP64 path only
    assert lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx)) == capi.ERR_UNSUPPORTED
    d = capi.default_desc()
    d.bc_kind[capi.XP] = 7  # not a boundary kind
    assert lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx)) == capi.ERR_ARG
    d = capi.default_desc()
    d.num_phases = 9
    assert lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx)) == capi.ERR_ARG
    assert lib.hydro_gpu_stencil_workspace_size(3, 8, 8, 8) > 8 * 8 * 8 * 7 * 8


def test_no_device_fails_loudly(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    d = capi.default_desc()
    ctx = ctypes.c_void_p()
    st = lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx))
    assert st == capi.ERR_NO_DEVICE
    from hydro_gb300.solver import Hydro
    with pytest.raises(capi.HydroError):
        Hydro(d)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(capi, "_LIB", None)
    monkeypatch.setattr(capi, "lib_path", lambda: str(tmp_path / "absent.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        capi.load()


def test_create_needs_opt_in_for_substituted_solvers(lib):
    """Solvers the GPU does not have (velocity LU, pressure Gauss-Seidel /
    Jacobi / LU) are an explicit request: without substitute_solvers the
    description is refused before any device work (no GPU needed)."""
    ctx = ctypes.c_void_p()
    for field, value in (("velocity_solver", capi.LINEAR_LU),
                         ("pressure_solver", capi.LINEAR_GAUSS_SEIDEL),
                         ("pressure_solver", capi.LINEAR_JACOBI),
                         ("pressure_solver", capi.LINEAR_LU)):
        d = capi.default_desc()
        setattr(d, field, value)
        assert lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx)) == capi.ERR_UNSUPPORTED
    d = capi.default_desc()
    d.velocity_solver = 17
    assert lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx)) == capi.ERR_ARG
    # with the opt-in the description passes validation (and without a GPU
    # here stops at the device check)
    d = capi.default_desc()
    d.velocity_solver = capi.LINEAR_LU
    d.substitute_solvers = 1
    st = lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx))
    assert st in (capi.ERR_NO_DEVICE, capi.OK)
    if st == capi.OK:
        lib.hydro_gpu_destroy(ctx)


def test_create_checks_one_group_solves(lib):
    """cta_threads / cta_cluster are validated before any device work: a
    thread count that is no multiple of 32, a cluster of 3 or a cluster
    without a thread count is HYDRO_ERR_ARG; FP64, a periodic direction or
    2^24 cells and more is HYDRO_ERR_UNSUPPORTED (the one-group passes index
    cells through FP32 reciprocals)."""
    torch = pytest.importorskip("torch")
    ctx = ctypes.c_void_p()

    def desc(nx, ny, **kw):
        d = capi.default_desc()
        d.dim = 2
        d.n[0], d.n[1], d.n[2] = nx, ny, 1
        d.precision = capi.MIXED
        d.pressure_solver = capi.LINEAR_MGCG
        d.cta_threads = 1024
        for k, v in kw.items():
            setattr(d, k, v)
        return d

    for kw in ({"cta_threads": 48}, {"cta_cluster": 3}, {"cta_threads": 0, "cta_cluster": 4}):
        d = desc(64, 64, **kw)
        assert lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx)) == capi.ERR_ARG, kw
    d = desc(64, 64, precision=capi.FP64)
    assert lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx)) == capi.ERR_UNSUPPORTED
    d = desc(64, 64)
    d.periodic[0] = 1
    assert lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx)) == capi.ERR_UNSUPPORTED
    d = desc(4096, 4096)  # 2^24 cells
    assert lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx)) == capi.ERR_UNSUPPORTED
    if not torch.cuda.is_available():
        # one cell fewer passes validation and stops at the device check
        d = desc(4096, 4095)
        assert lib.hydro_gpu_create(ctypes.byref(d), ctypes.byref(ctx)) == capi.ERR_NO_DEVICE
