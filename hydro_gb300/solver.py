"""Python host mirror of the reference's solver interface over the C-ABI.

``Hydro`` holds one GPU context (libhydro_gpu.so) and exposes the methods of
solver::FluidSolver (fluid.hpp:202-253) -- StartStep, MakeIteration,
FinishStep, IsConverged, GetConvergenceIndicator, GetIterationCount,
GetVelocity/GetPressure/GetVolumeFlux(layer), GetAutoTimeStep,
SetTimeStep -- plus AdvectionSolverMulti::GetField (advection.hpp:82) and
hydro<Mesh>::step / UpdateFluidProperties / CalcStat (hydro2d.hpp).
Errors raise ``capi.HydroError`` carrying the C status (HYDRO_ERR_NAN maps
the reference's ``throw std::string("NaN pressure")``, fluid.hpp:1164-1166).
"""
import ctypes

import numpy as np

from . import capi

Layers = {"time_curr": capi.TIME_CURR, "time_prev": capi.TIME_PREV,
          "iter_curr": capi.ITER_CURR, "iter_prev": capi.ITER_PREV}


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Hydro:
    prefix = "hydro_gpu"

    def __init__(self, desc, stream=None, _ctx=None):
        self.lib = capi.load()
        self.desc = desc.copy()
        if stream is not None:
            self.desc.stream = ctypes.c_void_p(stream)
        self._owned = _ctx is None
        if _ctx is None:
            self.ctx = ctypes.c_void_p()
            self._check(self.lib.hydro_gpu_create(ctypes.byref(self.desc),
                                                  ctypes.byref(self.ctx)), "hydro_gpu_create")
        else:
            self.ctx = _ctx
        self.nc = self.desc.ncells
        self.nf = self.desc.nfaces
        self.dim = self.desc.dim

    @staticmethod
    def _check(st, where):
        if st != capi.OK:
            raise capi.HydroError(st, where)

    def close(self):
        if getattr(self, "ctx", None):
            if getattr(self, "_owned", True):
                self.lib.hydro_gpu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        self.close()

    def _call(self, name, *args):
        self._check(getattr(self.lib, "hydro_gpu_" + name)(self.ctx, *args), "hydro_gpu_" + name)

    def _size(self, field):
        if field == capi.F_VOLUME_FLUX:
            return self.nf
        if field in capi.VECTOR_FIELDS:
            return self.nc * self.dim
        if field in (capi.F_PARTIAL_DENSITY, capi.F_VOLUME_FRACTION):
            return self.nc * self.desc.num_phases
        return self.nc

    # ---- fields
    def set_field(self, field, values, layer=capi.TIME_CURR):
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        self._call("set_field", field, layer, _dp(a), a.size)

    def get_field(self, field, layer=capi.TIME_CURR):
        a = np.empty(self._size(field), dtype=np.float64)
        self._call("get_field", field, layer, _dp(a), a.size)
        return a

    def field_ptr(self, field, layer=capi.TIME_CURR):
        p = ctypes.POINTER(ctypes.c_double)()
        self._call("field_ptr", field, layer, ctypes.byref(p))
        return ctypes.cast(p, ctypes.c_void_p).value

    def stream_ptr(self):
        """The context's cudaStream_t (hydro_gpu_get_stream)."""
        p = ctypes.c_void_p()
        self._call("get_stream", ctypes.byref(p))
        return p.value

    def GetVelocity(self, layer="time_curr"):
        return self.get_field(capi.F_VELOCITY, Layers[layer]).reshape(self.dim, self.nc)

    def GetPressure(self, layer="time_curr"):
        return self.get_field(capi.F_PRESSURE, Layers[layer])

    def GetVolumeFlux(self, layer="time_curr"):
        return self.get_field(capi.F_VOLUME_FLUX, Layers[layer])

    def GetField(self, phase):
        return self.get_field(capi.F_PARTIAL_DENSITY).reshape(-1, self.nc)[phase]

    # ---- lifecycle
    def init_state(self):
        self._call("init_state")

    def update_properties(self):
        self._call("update_properties")

    def start_step(self):
        self._call("start_step")

    def make_iteration(self):
        self._call("make_iteration")

    def finish_step(self):
        self._call("finish_step")

    StartStep = start_step
    MakeIteration = make_iteration
    FinishStep = finish_step
    UpdateFluidProperties = update_properties

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

    GetConvergenceIndicator = convergence_indicator
    GetIterationCount = iteration_count
    IsConverged = is_converged

    def auto_time_step(self):
        v = ctypes.c_double()
        self._call("get_auto_time_step", ctypes.byref(v))
        return v.value

    GetAutoTimeStep = auto_time_step

    def set_time_step(self, dt, dta):
        self._call("set_time_step", dt, dta)

    def time(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._call("get_time", ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def advection_step(self):
        n = ctypes.c_int()
        self._call("advection_step", ctypes.byref(n))
        return n.value

    @staticmethod
    def _check_step(st, where):
        # HYDRO_NOT_CONVERGED: the step is complete, a pressure solve stopped
        # at its iteration limit (the reference goes on past a solver's limit
        # too); the stats carry the status and the count of such solves
        if st not in (capi.OK, capi.NOT_CONVERGED):
            raise capi.HydroError(st, where)

    def step(self):
        """One time step (hydro_gpu_step); returns its stats.  A step in
        which a pressure solve stopped at its limit returns normally with
        ``status`` HYDRO_NOT_CONVERGED; every other error raises."""
        st = capi.StepStats()
        self._check_step(self.lib.hydro_gpu_step(self.ctx, ctypes.byref(st)), "hydro_gpu_step")
        return st.as_dict()

    def step_graph(self):
        """The same step as one CUDA-graph launch (hydro_gpu_step_graph)."""
        st = capi.StepStats()
        self._check_step(self.lib.hydro_gpu_step_graph(self.ctx, ctypes.byref(st)),
                         "hydro_gpu_step_graph")
        return st.as_dict()

    def calc_stat(self):
        s = capi.Stat()
        self._call("calc_stat", ctypes.byref(s))
        return s

    # ---- temperature (HeatSolver, heat.hpp:18-94)
    def heat_create(self, heat):
        """Attach the temperature equation (hydro_gpu_heat_create); every
        step then advances it once after advection."""
        self.heat = capi.HeatDesc.from_buffer_copy(heat)
        self._call("heat_create", ctypes.byref(self.heat))

    def heat_step(self):
        self._call("heat_step")

    def temperature(self, layer=capi.TIME_CURR):
        return self.get_field(capi.F_TEMPERATURE, layer)

    GetTemperature = temperature

    # ---- measurement hooks
    def set_profiling(self, on):
        self._call("set_profiling", 1 if on else 0)

    def reset_profile(self):
        self._call("reset_profile")

    def profile(self):
        out = {}
        for g, name in enumerate(capi.PROF_GROUPS):
            n = ctypes.c_longlong()
            ms = ctypes.c_double()
            self._call("get_profile", g, ctypes.byref(n), ctypes.byref(ms))
            if n.value:
                out[name] = (n.value, ms.value)
        return out


def launch_count():
    n = ctypes.c_longlong()
    capi.load().hydro_gpu_get_launch_count(ctypes.byref(n))
    return n.value


class Batch:
    """Independent cases advanced together, one CUDA-graph launch per batch
    step (hydro_gpu_batch_*).  ``cases[i]`` is a ``Hydro`` view of case i
    (fields, stats) owned by the batch."""

    def __init__(self, descs):
        self.lib = capi.load()
        arr = (capi.HydroDesc * len(descs))()
        for i, d in enumerate(descs):
            arr[i] = d.copy()
        self.b = ctypes.c_void_p()
        Hydro._check(self.lib.hydro_gpu_batch_create(arr, len(descs), ctypes.byref(self.b)),
                     "hydro_gpu_batch_create")
        self.cases = []
        for i, d in enumerate(descs):
            c = ctypes.c_void_p()
            Hydro._check(self.lib.hydro_gpu_batch_case(self.b, i, ctypes.byref(c)),
                         "hydro_gpu_batch_case")
            self.cases.append(Hydro(d, _ctx=c))

    def init_state(self):
        Hydro._check(self.lib.hydro_gpu_batch_init_state(self.b), "hydro_gpu_batch_init_state")

    def step(self):
        st = (capi.StepStats * len(self.cases))()
        Hydro._check_step(self.lib.hydro_gpu_batch_step(self.b, st), "hydro_gpu_batch_step")
        return [s.as_dict() for s in st]

    def close(self):
        if getattr(self, "b", None):
            for c in self.cases:
                c.ctx = None
            self.lib.hydro_gpu_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        self.close()


def make(desc, u0, q0, stream=None):
    """Create a context, upload the initial velocity and partial densities
    and compute the initial fluxes and properties."""
    h = Hydro(desc, stream=stream)
    h.set_field(capi.F_VELOCITY, u0)
    h.set_field(capi.F_PARTIAL_DENSITY, q0)
    h.init_state()
    return h


def stencil_solve(dim, n, face_coeff, shift, pinned_cell, pinned_value, rhs, tol, limit, x0=None):
    """hydro_gpu_stencil_solve on host numpy arrays; device buffers come from
    torch (plumbing only), the solve itself is the library's."""
    import torch
    lib = capi.load()
    nz = n[2] if dim == 3 else 1
    nc = n[0] * n[1] * nz
    ws_bytes = lib.hydro_gpu_stencil_workspace_size(dim, n[0], n[1], nz)
    dev = torch.device("cuda")
    dk = torch.from_numpy(np.ascontiguousarray(face_coeff, dtype=np.float64)).to(dev)
    dr = torch.from_numpy(np.ascontiguousarray(rhs, dtype=np.float64)).to(dev)
    x_init = np.zeros(nc) if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
    dx = torch.from_numpy(x_init).to(dev)
    dw = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    it = ctypes.c_int()
    res = ctypes.c_double()
    st = lib.hydro_gpu_stencil_solve(dim, n[0], n[1], nz, dk.data_ptr(), shift, pinned_cell,
                                     pinned_value, dr.data_ptr(), dx.data_ptr(),
                                     0 if x0 is None else 1, tol, limit, dw.data_ptr(), None,
                                     ctypes.byref(it), ctypes.byref(res))
    torch.cuda.synchronize()
    return st, dx.cpu().numpy(), it.value, res.value
