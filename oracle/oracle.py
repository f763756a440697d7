"""ctypes wrapper of the CPU oracle (oracle/liboracle.so) and of the
reference harness (oracle/_ref/libhydro_ref.so, present only where the
reference tree was available at build time).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py, as the checker or baseline.
"""
import ctypes
import os
import subprocess

import numpy as np

from hydro_gb300 import capi

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libhydro_ref.so")

_oracle = None
_ref = None


def build(ref=True):
    """make -C oracle (the _ref part only when the reference tree exists)."""
    target = "all" if ref else "liboracle.so"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)


def lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_LIB):
            build(ref=False)
        _oracle = ctypes.CDLL(ORACLE_LIB)
        capi._declare(_oracle, "oracle")
        _oracle.oracle_smooth_field.argtypes = [ctypes.c_void_p,
                                                ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        _oracle.oracle_smooth_field.restype = ctypes.c_int
        _oracle.oracle_set_threads.argtypes = [ctypes.c_int]
        _oracle.oracle_set_threads.restype = ctypes.c_int
        _oracle.oracle_heat_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(capi.HeatDesc)]
        _oracle.oracle_heat_create.restype = ctypes.c_int
        _oracle.oracle_heat_get_temperature.argtypes = [ctypes.c_void_p,
                                                        ctypes.POINTER(ctypes.c_double),
                                                        ctypes.c_size_t]
        _oracle.oracle_heat_get_temperature.restype = ctypes.c_int
    return _oracle


def ref_available():
    return os.path.exists(REF_LIB)


_ref_variants = {}


def ref_lib(variant=""):
    """The reference harness; variant "perx" / "perxz" is the build with the
    reference's compile-time periodicity switches PERX / PERX+PERZ."""
    global _ref
    if variant:
        if variant not in _ref_variants:
            lib = ctypes.CDLL(REF_LIB.replace(".so", "_%s.so" % variant))
            D = ctypes.POINTER(ctypes.c_double)
            lib.ref_run.argtypes = [ctypes.POINTER(capi.HydroDesc), D, D, ctypes.c_int,
                                    D, D, D, D, ctypes.POINTER(capi.StepStats)]
            lib.ref_run.restype = ctypes.c_int
            lib.ref_run_heat.argtypes = [ctypes.POINTER(capi.HydroDesc),
                                         ctypes.POINTER(capi.HeatDesc), D, D, ctypes.c_int,
                                         D, D, D, D, D, ctypes.POINTER(capi.StepStats)]
            lib.ref_run_heat.restype = ctypes.c_int
            _ref_variants[variant] = lib
        return _ref_variants[variant]
    if _ref is None:
        _ref = ctypes.CDLL(REF_LIB)
        D = ctypes.POINTER(ctypes.c_double)
        _ref.ref_run.argtypes = [ctypes.POINTER(capi.HydroDesc), D, D, ctypes.c_int,
                                 D, D, D, D, ctypes.POINTER(capi.StepStats)]
        _ref.ref_run.restype = ctypes.c_int
        _ref.ref_smooth.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), D, ctypes.c_int]
        _ref.ref_smooth.restype = ctypes.c_int
        _ref.ref_run_heat.argtypes = [ctypes.POINTER(capi.HydroDesc),
                                      ctypes.POINTER(capi.HeatDesc), D, D, ctypes.c_int,
                                      D, D, D, D, D, ctypes.POINTER(capi.StepStats)]
        _ref.ref_run_heat.restype = ctypes.c_int
        C = ctypes.c_char_p
        _ref.ref_write_vts.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), D, D,
                                       ctypes.c_int, ctypes.POINTER(C), ctypes.POINTER(D),
                                       ctypes.c_int, ctypes.POINTER(C), ctypes.POINTER(D), C,
                                       ctypes.c_int, D]
        _ref.ref_write_vts.restype = ctypes.c_int
    return _ref


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(st, where):
    if st != capi.OK:
        raise capi.HydroError(st, where)


class Oracle:
    """Same method set as hydro_gb300.solver.Hydro, computed on the CPU."""

    prefix = "oracle"

    def __init__(self, desc, threads=1):
        self.lib = lib()
        self.lib.oracle_set_threads(threads)
        self.desc = desc.copy()
        self.ctx = ctypes.c_void_p()
        _check(self.lib.oracle_create(ctypes.byref(self.desc), ctypes.byref(self.ctx)),
               "oracle_create")
        self.nc = self.desc.ncells
        self.nf = self.desc.nfaces
        self.dim = self.desc.dim

    def __del__(self):
        if getattr(self, "ctx", None):
            self.lib.oracle_destroy(self.ctx)
            self.ctx = None

    def _call(self, name, *args):
        _check(getattr(self.lib, "oracle_" + name)(self.ctx, *args), "oracle_" + name)

    def _size(self, field):
        if field == capi.F_VOLUME_FLUX:
            return self.nf
        if field in capi.VECTOR_FIELDS:
            return self.nc * self.dim
        if field in (capi.F_PARTIAL_DENSITY, capi.F_VOLUME_FRACTION):
            return self.nc * self.desc.num_phases
        return self.nc

    def set_field(self, field, values, layer=capi.TIME_CURR):
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        self._call("set_field", field, layer, _dp(a), a.size)

    def get_field(self, field, layer=capi.TIME_CURR):
        a = np.empty(self._size(field), dtype=np.float64)
        self._call("get_field", field, layer, _dp(a), a.size)
        return a

    def init_state(self):
        self._call("init_state")

    def step(self):
        st = capi.StepStats()
        self._call("step", ctypes.byref(st))
        return st.as_dict()

    def start_step(self):
        self._call("start_step")

    def make_iteration(self):
        self._call("make_iteration")

    def finish_step(self):
        self._call("finish_step")

    def update_properties(self):
        self._call("update_properties")

    def advection_step(self):
        n = ctypes.c_int()
        self._call("advection_step", ctypes.byref(n))
        return n.value

    def convergence_indicator(self):
        v = ctypes.c_double()
        self._call("get_convergence_indicator", ctypes.byref(v))
        return v.value

    def iteration_count(self):
        v = ctypes.c_int()
        self._call("get_iteration_count", ctypes.byref(v))
        return v.value

    def is_converged(self):
        v = ctypes.c_int()
        self._call("is_converged", ctypes.byref(v))
        return bool(v.value)

    def auto_time_step(self):
        v = ctypes.c_double()
        self._call("get_auto_time_step", ctypes.byref(v))
        return v.value

    def set_time_step(self, dt, dta):
        self._call("set_time_step", dt, dta)

    def time(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._call("get_time", ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def calc_stat(self):
        s = capi.Stat()
        self._call("calc_stat", ctypes.byref(s))
        return s

    def heat_create(self, heat):
        self.heat = capi.HeatDesc.from_buffer_copy(heat)
        self._call("heat_create", ctypes.byref(self.heat))

    def temperature(self):
        a = np.empty(self.nc, dtype=np.float64)
        self._call("heat_get_temperature", _dp(a), a.size)
        return a

    def smooth(self, field, repeat):
        a = np.ascontiguousarray(field, dtype=np.float64).copy()
        self._call("smooth_field", _dp(a), repeat)
        return a


def stencil_solve(dim, n, face_coeff, shift, pinned_cell, pinned_value, rhs, tol,
                  limit, x0=None):
    L = lib()
    x = np.zeros(int(np.prod(n[:dim])), dtype=np.float64) if x0 is None else x0.copy()
    fc = np.ascontiguousarray(face_coeff, dtype=np.float64)
    b = np.ascontiguousarray(rhs, dtype=np.float64)
    it = ctypes.c_int()
    res = ctypes.c_double()
    nz = n[2] if dim == 3 else 1
    st = L.oracle_stencil_solve(dim, n[0], n[1], nz, _dp(fc), shift, pinned_cell,
                                pinned_value, _dp(b), _dp(x), 0 if x0 is None else 1,
                                tol, limit, ctypes.byref(it), ctypes.byref(res))
    return st, x, it.value, res.value


def _ref_for(desc):
    """Harness build for the case's periodic directions: x selects PERX,
    x and z (3D) PERX+PERZ."""
    per = tuple(bool(desc.periodic[k]) for k in range(3))
    variants = {(False, False, False): "", (True, False, False): "perx",
                (True, False, True): "perxz"}
    if desc.dim == 2:
        per = (per[0], per[1], False)
    if per not in variants:
        raise ValueError("the reference switches periodicity on x (PERX) and x+z (PERZ) only")
    return ref_lib(variants[per])


def ref_run(desc, u0, q0, nsteps, variant=None):
    """Run the reference's own FluidSimple + AdvectionSolverMultiExplicit for
    nsteps steps; returns (u, p, F, q, stats list).  Periodic directions x
    (and z in 3D) select the harness built with PERX (PERZ).  variant
    "adapter": the harness with the reference-side adapter classes in their
    place, the C-ABI forwarded to this oracle (oracle/adapter_shim.c)."""
    R = ref_lib(variant) if variant else _ref_for(desc)
    nc, nf, dim = desc.ncells, desc.nfaces, desc.dim
    nph = desc.num_phases
    u0 = np.ascontiguousarray(u0, dtype=np.float64).ravel()
    q0 = np.ascontiguousarray(q0, dtype=np.float64).ravel()
    u = np.empty(nc * dim)
    p = np.empty(nc)
    F = np.empty(nf)
    q = np.empty(nc * nph)
    stats = (capi.StepStats * max(nsteps, 1))()
    d = desc.copy()
    st = R.ref_run(ctypes.byref(d), _dp(u0), _dp(q0), nsteps, _dp(u), _dp(p), _dp(F),
                   _dp(q), stats)
    _check(st, "ref_run")
    return u, p, F, q, [stats[i].as_dict() for i in range(nsteps)]


def ref_run_heat(desc, heat, u0, q0, nsteps):
    """ref_run with the reference's HeatSolver attached (hydro2d.hpp:650-687,
    1607-1613); returns (u, p, F, q, T, stats list)."""
    R = _ref_for(desc)
    nc, nf, dim, nph = desc.ncells, desc.nfaces, desc.dim, desc.num_phases
    u0 = np.ascontiguousarray(u0, dtype=np.float64).ravel()
    q0 = np.ascontiguousarray(q0, dtype=np.float64).ravel()
    u, p, F, q, T = (np.empty(nc * dim), np.empty(nc), np.empty(nf), np.empty(nc * nph),
                     np.empty(nc))
    stats = (capi.StepStats * max(nsteps, 1))()
    d, h = desc.copy(), capi.HeatDesc.from_buffer_copy(heat)
    _check(R.ref_run_heat(ctypes.byref(d), ctypes.byref(h), _dp(u0), _dp(q0), nsteps, _dp(u),
                          _dp(p), _dp(F), _dp(q), _dp(T), stats), "ref_run_heat")
    return u, p, F, q, T, [stats[i].as_dict() for i in range(nsteps)]


def ref_write_vts(dim, n, lo, hi, node_fields, cell_fields, base, times):
    """Frames written by the reference's own ParaView session
    (output_paraview.hpp) for the given {name: array} node and cell entries;
    one frame per entry of `times`, files <base>.<k>.vts and <base>.pvd."""
    R = ref_lib()
    C = ctypes.c_char_p

    def pack(fields):
        names = (C * max(1, len(fields)))(*[k.encode() for k in fields])
        arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in fields.values()]
        ptrs = (ctypes.POINTER(ctypes.c_double) * max(1, len(arrs)))(*[_dp(a) for a in arrs])
        return names, ptrs, arrs

    nn, nptr, keep1 = pack(node_fields)
    cn, cptr, keep2 = pack(cell_fields)
    t = np.ascontiguousarray(times, dtype=np.float64)
    _check(R.ref_write_vts(dim, (ctypes.c_int * 3)(*n), _dp(np.asarray(lo, dtype=np.float64)),
                           _dp(np.asarray(hi, dtype=np.float64)), len(node_fields), nn, nptr,
                           len(cell_fields), cn, cptr, base.encode(), len(t), _dp(t)),
           "ref_write_vts")
    del keep1, keep2


def ref_smooth(dim, n, field, repeat):
    R = ref_lib()
    a = np.ascontiguousarray(field, dtype=np.float64).copy()
    nn = (ctypes.c_int * 3)(*n)
    _check(R.ref_smooth(dim, nn, _dp(a), repeat), "ref_smooth")
    return a
