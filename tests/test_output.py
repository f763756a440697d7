"""Output in the reference's file formats.  The .vts frames written from
host arrays match, byte for byte, the frames the reference's own ParaView
session (output_paraview.hpp) wrote for the same arrays (tests/golden/vts*,
made by tests/golden/make_golden.py); no GPU is needed for that path."""
import ctypes
import os

import numpy as np
import pytest

from hydro_gb300 import capi

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden(name):
    return np.load(os.path.join(HERE, "golden", name + ".npz"), allow_pickle=False)


@pytest.mark.parametrize("name", ["vts2d", "vts3d"])
def test_host_frames_match_reference_writer(built, tmp_path, name):
    g = _golden(name)
    lib = capi.load()
    entries = [(str(k), 1, g["node_" + str(k)]) for k in g["node_names"]]
    entries += [(str(k), 0, g["cell_" + str(k)]) for k in g["cell_names"]]
    names = (ctypes.c_char_p * len(entries))(*[e[0].encode() for e in entries])
    on_nodes = (ctypes.c_int * len(entries))(*[e[1] for e in entries])
    arrs = [np.ascontiguousarray(e[2], dtype=np.float64) for e in entries]
    data = (ctypes.POINTER(ctypes.c_double) * len(arrs))(
        *[a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in arrs])
    n = (ctypes.c_int * 3)(*[int(v) for v in g["n"]])
    lo = np.ascontiguousarray(g["lo"], dtype=np.float64)
    hi = np.ascontiguousarray(g["hi"], dtype=np.float64)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    for k, frame in enumerate(g["frames"]):
        path = tmp_path / ("f%d.vts" % k)
        st = lib.hydro_vts_write_host(str(path).encode(), int(g["dim"]), n, dp(lo), dp(hi),
                                      len(entries), names, on_nodes, data)
        assert st == capi.OK
        assert path.read_text() == str(frame)


def test_unwritable_path_reports_io_error(built):
    lib = capi.load()
    st = lib.hydro_vts_write_host(b"/nonexistent/dir/x.vts", 2, (ctypes.c_int * 3)(2, 2, 1),
                                  (ctypes.c_double * 3)(0, 0, 0), (ctypes.c_double * 3)(1, 1, 1),
                                  0, None, None, None)
    assert st == capi.ERR_IO


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["vts2d", "vts3d"])
def test_async_writer_matches_reference_writer(built, tmp_path, name, monkeypatch):
    """The context-bound writer (pinned copies on a side stream, formatting
    on a worker thread) writes the same bytes as the reference for fields set
    on a context, frames and collection included."""
    from hydro_gb300.solver import Hydro
    g = _golden(name)
    dim = int(g["dim"])
    d = capi.default_desc()
    d.dim = dim
    for k in range(3):
        d.n[k] = int(g["n"][k]) if k < dim else 1
        d.lo[k] = float(g["lo"][k])
        d.hi[k] = float(g["hi"][k])
    d.num_phases = 2
    d.advection_enable = 0
    h = Hydro(d)
    nc = d.ncells
    u = np.concatenate([g["cell_velocity_" + c] for c in "xyz"[:dim]])
    q0 = np.concatenate([g["cell_volume_fraction_0"], g["cell_volume_fraction_1"]])
    h.set_field(capi.F_VELOCITY, np.zeros(nc * dim))
    h.set_field(capi.F_PARTIAL_DENSITY, q0)
    h.init_state()
    h.set_field(capi.F_VELOCITY, u)
    h.set_field(capi.F_PRESSURE, g["cell_pressure"])
    h.set_field(capi.F_VOLUME_FRACTION, q0)
    monkeypatch.chdir(tmp_path)
    lib = capi.load()
    out = ctypes.c_void_p()
    fields = ",".join([str(k) for k in g["node_names"]] + [str(k) for k in g["cell_names"]])
    assert lib.hydro_output_open(h.ctx, (name + ".field").encode(), fields.encode(),
                                 ctypes.byref(out)) == capi.OK
    for t in g["times"]:
        assert lib.hydro_output_write(out, float(t)) == capi.OK
    assert lib.hydro_output_close(out) == capi.OK
    for k, frame in enumerate(g["frames"]):
        assert (tmp_path / ("%s.field.%d.vts" % (name, k))).read_text() == str(frame)
    assert (tmp_path / (name + ".field.pvd")).read_text() == str(g["pvd"])
    h.close()
