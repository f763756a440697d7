"""ctypes mirror of include/hydro_gpu.h and the loader of libhydro_gpu.so.

The structures here are the C-ABI's own layout; the library is the CUDA
implementation built by ``hydro_gb300.build`` (nvcc, sm_103a) next to this
file.  Loading fails loudly when the library is missing: there is no CPU
fallback behind this interface.
"""
import ctypes
import os

HYDRO_MAX_PHASES = 4

# enum hydro_status
(OK, ERR_ARG, ERR_CUDA, ERR_NAN, NOT_CONVERGED, ERR_UNSUPPORTED, ERR_NOMEM, ERR_NO_DEVICE,
 ERR_IO) = range(9)
STATUS_NAMES = {
    OK: "HYDRO_OK", ERR_ARG: "HYDRO_ERR_ARG", ERR_CUDA: "HYDRO_ERR_CUDA",
    ERR_NAN: "HYDRO_ERR_NAN", NOT_CONVERGED: "HYDRO_NOT_CONVERGED",
    ERR_UNSUPPORTED: "HYDRO_ERR_UNSUPPORTED", ERR_NOMEM: "HYDRO_ERR_NOMEM",
    ERR_NO_DEVICE: "HYDRO_ERR_NO_DEVICE",
    ERR_IO: "HYDRO_ERR_IO",
}

# enum hydro_side
XM, XP, YM, YP, ZM, ZP = range(6)
# enum hydro_bc_kind
BC_WALL, BC_INLET, BC_OUTLET = range(3)
# enum hydro_linear
LINEAR_GAUSS_SEIDEL, LINEAR_JACOBI, LINEAR_CG, LINEAR_LU, LINEAR_MGCG = range(5)
LINEAR_NAMES = {"gauss_seidel": LINEAR_GAUSS_SEIDEL, "jacobi": LINEAR_JACOBI,
                "cg": LINEAR_CG, "lu": LINEAR_LU, "mgcg": LINEAR_MGCG}
# enum hydro_precision
FP64, MIXED = range(2)
# enum hydro_field
(F_VELOCITY, F_PRESSURE, F_VOLUME_FLUX, F_PARTIAL_DENSITY, F_VOLUME_FRACTION,
 F_DENSITY, F_VISCOSITY, F_FORCE, F_VOLUME_SOURCE, F_MASS_SOURCE,
 F_PRESSURE_CORRECTION, F_DIAG_COEFF, F_SURFACE_FORCE, F_TEMPERATURE,
 F_CONDUCTIVITY, F_PRESSURE_RHS) = range(16)
VECTOR_FIELDS = (F_VELOCITY, F_FORCE, F_SURFACE_FORCE)
# enum hydro_layer (solver::Layers order)
TIME_CURR, TIME_PREV, ITER_CURR, ITER_PREV = range(4)
# enum hydro_prof_group
PROF_GROUPS = ["vel_grad", "force", "mom_assemble", "mom_sweep", "rhie_chow", "pressure_rhs",
               "cg_init", "cg_spmv", "cg_update", "cg_dir", "ir_residual", "correct",
               "adv_faces", "adv_update", "props", "mg_vcycle", "other", "guess"]


class HydroDesc(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("n", ctypes.c_int * 3),
        ("lo", ctypes.c_double * 3),
        ("hi", ctypes.c_double * 3),
        ("bc_kind", ctypes.c_int * 6),
        ("bc_velocity", (ctypes.c_double * 3) * 6),
        ("dt", ctypes.c_double),
        ("dt_auto", ctypes.c_int),
        ("cfl", ctypes.c_double),
        ("cfl_advection", ctypes.c_double),
        ("dt_max", ctypes.c_double),
        ("velocity_relaxation_factor", ctypes.c_double),
        ("pressure_relaxation_factor", ctypes.c_double),
        ("rhie_chow_factor", ctypes.c_double),
        ("time_second_order", ctypes.c_int),
        ("force_geometric_average", ctypes.c_int),
        ("guess_extrapolation", ctypes.c_double),
        ("meshvel", ctypes.c_double * 3),
        ("convergence_tolerance", ctypes.c_double),
        ("num_iterations_limit", ctypes.c_int),
        ("simpler", ctypes.c_int),
        ("velocity_solver", ctypes.c_int),
        ("velocity_tolerance", ctypes.c_double),
        ("velocity_iters_limit", ctypes.c_int),
        ("velocity_omega", ctypes.c_double),
        ("pressure_solver", ctypes.c_int),
        ("pressure_tolerance", ctypes.c_double),
        ("pressure_iters_limit", ctypes.c_int),
        ("pressure_omega", ctypes.c_double),
        ("precision", ctypes.c_int),
        ("pressure_fixed_cell", ctypes.c_int),
        ("pressure_fixed_value", ctypes.c_double),
        ("num_phases", ctypes.c_int),
        ("density", ctypes.c_double * HYDRO_MAX_PHASES),
        ("viscosity", ctypes.c_double * HYDRO_MAX_PHASES),
        ("gravity", ctypes.c_double * 3),
        ("force", ctypes.c_double * 3),
        ("sigma", ctypes.c_double),
        ("density_smooth_times", ctypes.c_int),
        ("viscosity_smooth_times", ctypes.c_int),
        ("force_smooth_times", ctypes.c_int),
        ("advection_enable", ctypes.c_int),
        ("advection_dt_factor", ctypes.c_double),
        ("tvd_split", ctypes.c_int),
        ("sharp", ctypes.c_double),
        ("stream", ctypes.c_void_p),
        ("periodic", ctypes.c_int * 3),
        ("rigid_box", ctypes.c_int),
        ("rigid_box_lo", ctypes.c_double * 3),
        ("rigid_box_hi", ctypes.c_double * 3),
        ("substitute_solvers", ctypes.c_int),
        ("cta_threads", ctypes.c_int),
        ("cta_cluster", ctypes.c_int),
    ]

    @property
    def ncells(self):
        n = 1
        for d in range(self.dim):
            n *= self.n[d]
        return n

    @property
    def nfaces(self):
        tot = 0
        for d in range(self.dim):
            c = 1
            for e in range(self.dim):
                c *= self.n[e] + (1 if e == d else 0)
            tot += c
        return tot

    def copy(self):
        other = HydroDesc()
        ctypes.memmove(ctypes.byref(other), ctypes.byref(self), ctypes.sizeof(HydroDesc))
        return other


class StepStats(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int),
        ("outer_iterations", ctypes.c_int),
        ("convergence_indicator", ctypes.c_double),
        ("velocity_sweeps", ctypes.c_int),
        ("pressure_iterations", ctypes.c_int),
        ("pressure_residual", ctypes.c_double),
        ("advection_substeps", ctypes.c_int),
        ("dt", ctypes.c_double),
        ("dt_advection", ctypes.c_double),
        ("time", ctypes.c_double),
        ("pressure_unconverged", ctypes.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class HeatDesc(ctypes.Structure):
    _fields_ = [
        ("temperature_initial", ctypes.c_double),
        ("conductivity", ctypes.c_double * HYDRO_MAX_PHASES),
        ("box_lo", ctypes.c_double * 3),
        ("box_hi", ctypes.c_double * 3),
        ("box_temperature", ctypes.c_double),
        ("relaxation_factor", ctypes.c_double),
        ("time_second_order", ctypes.c_int),
        ("solver", ctypes.c_int),
        ("tolerance", ctypes.c_double),
        ("iters_limit", ctypes.c_int),
        ("dt", ctypes.c_double),
    ]


def heat_to_dict(h):
    out = {}
    for name, _ in HeatDesc._fields_:
        v = getattr(h, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


def heat_from_dict(dct):
    h = HeatDesc()
    for name, v in dct.items():
        if isinstance(v, list):
            arr = getattr(h, name)
            for i, e in enumerate(v):
                arr[i] = e
        else:
            setattr(h, name, v)
    return h


def default_heat_desc(dt):
    """examples/general.hydroconf:80-91 (heat_relaxation_factor 1,
    time_second_order_heat 1), Jacobi sweeps to 1e-12, the given dt."""
    h = HeatDesc()
    h.relaxation_factor = 1.0
    h.time_second_order = 1
    h.solver = LINEAR_JACOBI
    h.tolerance = 1e-12
    h.iters_limit = 10000
    h.dt = dt
    return h


class Stat(ctypes.Structure):
    _fields_ = [
        ("volume", ctypes.c_double * HYDRO_MAX_PHASES),
        ("mass", ctypes.c_double * HYDRO_MAX_PHASES),
        ("pd_min", ctypes.c_double * HYDRO_MAX_PHASES),
        ("pd_max", ctypes.c_double * HYDRO_MAX_PHASES),
        ("center", (ctypes.c_double * 3) * HYDRO_MAX_PHASES),
        ("velocity", (ctypes.c_double * 3) * HYDRO_MAX_PHASES),
        ("partial_mass", ctypes.c_double * HYDRO_MAX_PHASES),
        ("volume_flux_in", ctypes.c_double * HYDRO_MAX_PHASES),
        ("volume_flux_out", ctypes.c_double * HYDRO_MAX_PHASES),
    ]


def default_desc():
    """Defaults of examples/general.hydroconf for the in-scope keys
    (the same values hydro_desc_default() writes)."""
    d = HydroDesc()
    d.dim = 2
    d.n[0], d.n[1], d.n[2] = 100, 100, 5
    for k in range(3):
        d.lo[k], d.hi[k] = 0.0, 1.0
    for s in range(6):
        d.bc_kind[s] = BC_WALL
        for k in range(3):
            d.bc_velocity[s][k] = 0.0
    d.dt = 0.01
    d.dt_auto = 0
    d.cfl = 0.5
    d.cfl_advection = 0.5
    d.dt_max = 0.0
    d.velocity_relaxation_factor = 0.8
    d.pressure_relaxation_factor = 0.9
    d.rhie_chow_factor = 1.0
    d.time_second_order = 1
    d.force_geometric_average = 0
    d.guess_extrapolation = 0.0
    d.convergence_tolerance = 1e-2
    d.num_iterations_limit = 10
    d.simpler = 0
    d.velocity_solver = LINEAR_JACOBI
    d.velocity_tolerance = 1e-3
    d.velocity_iters_limit = 1000
    d.velocity_omega = 1.0
    d.pressure_solver = LINEAR_CG
    d.pressure_tolerance = 1e-8
    d.pressure_iters_limit = 100000
    d.pressure_omega = 1.0
    d.precision = FP64
    d.pressure_fixed_cell = -1
    d.pressure_fixed_value = 0.0
    d.num_phases = 1
    for i in range(HYDRO_MAX_PHASES):
        d.density[i] = 1.0
        d.viscosity[i] = 1.0
    d.sigma = 0.0
    d.density_smooth_times = 2
    d.viscosity_smooth_times = 2
    d.force_smooth_times = 0
    d.advection_enable = 1
    d.advection_dt_factor = 0.1
    d.tvd_split = 0
    d.sharp = 0.0
    d.stream = None
    return d


class HydroError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        super().__init__("%s failed: %s" % (where, STATUS_NAMES.get(status, status)))


_LIB = None
LIB_NAME = "libhydro_gpu.so"


def lib_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), LIB_NAME)


def load():
    """Load the CUDA library (built in-tree).  Raises if it is absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(
            "%s not found: build it with hydro_gb300.build.build() "
            "(nvcc, sm_103a); the solver has no CPU fallback" % path)
    lib = ctypes.CDLL(path)
    _declare(lib, "hydro_gpu")
    _LIB = lib
    return lib


def _declare(lib, prefix):
    """Argument types shared by the GPU library and the oracle library."""
    P = ctypes.c_void_p
    D = ctypes.POINTER(ctypes.c_double)
    I = ctypes.c_int
    sig = {
        "create": [ctypes.POINTER(HydroDesc), ctypes.POINTER(P)],
        "destroy": [P],
        "set_field": [P, I, I, D, ctypes.c_size_t],
        "get_field": [P, I, I, D, ctypes.c_size_t],
        "init_state": [P],
        "update_properties": [P],
        "start_step": [P],
        "make_iteration": [P],
        "finish_step": [P],
        "get_convergence_indicator": [P, D],
        "get_iteration_count": [P, ctypes.POINTER(I)],
        "is_converged": [P, ctypes.POINTER(I)],
        "get_auto_time_step": [P, D],
        "set_time_step": [P, ctypes.c_double, ctypes.c_double],
        "get_time": [P, D, D],
        "advection_step": [P, ctypes.POINTER(I)],
        "advection_substep": [P],
        "step": [P, ctypes.POINTER(StepStats)],
        "calc_stat": [P, ctypes.POINTER(Stat)],
    }
    for name, args in sig.items():
        fn = getattr(lib, "%s_%s" % (prefix, name))
        fn.argtypes = args
        fn.restype = I
    stencil = getattr(lib, "%s_stencil_solve" % prefix)
    if prefix == "hydro_gpu":
        stencil.argtypes = [I, I, I, I, P, ctypes.c_double, ctypes.c_long,
                            ctypes.c_double, P, P, I, ctypes.c_double, I, P, P,
                            ctypes.POINTER(I), D]
        lib.hydro_gpu_stencil_workspace_size.argtypes = [I, I, I, I]
        lib.hydro_gpu_stencil_workspace_size.restype = ctypes.c_size_t
        lib.hydro_gpu_stencil_solve_noalloc.argtypes = [
            I, I, I, I, P, ctypes.c_double, ctypes.c_long, ctypes.c_double, P, P, I,
            ctypes.c_double, I, P, ctypes.POINTER(I), D]
        lib.hydro_gpu_stencil_solve_noalloc.restype = I
        lib.hydro_gpu_field_ptr.argtypes = [P, I, I, ctypes.POINTER(D)]
        lib.hydro_gpu_field_ptr.restype = I
        lib.hydro_desc_default.argtypes = [ctypes.POINTER(HydroDesc)]
        lib.hydro_desc_default.restype = I
        lib.hydro_gpu_set_profiling.argtypes = [P, I]
        lib.hydro_gpu_set_profiling.restype = I
        lib.hydro_gpu_reset_profile.argtypes = [P]
        lib.hydro_gpu_reset_profile.restype = I
        lib.hydro_gpu_get_profile.argtypes = [P, I, ctypes.POINTER(ctypes.c_longlong), D]
        lib.hydro_gpu_get_profile.restype = I
        lib.hydro_gpu_get_launch_count.argtypes = [ctypes.POINTER(ctypes.c_longlong)]
        lib.hydro_gpu_get_launch_count.restype = I
        lib.hydro_gpu_step_graph.argtypes = [P, ctypes.POINTER(StepStats)]
        lib.hydro_gpu_step_graph.restype = I
        batch = {
            "batch_create": [ctypes.POINTER(HydroDesc), I, ctypes.POINTER(P)],
            "batch_destroy": [P],
            "batch_size": [P, ctypes.POINTER(I)],
            "batch_case": [P, I, ctypes.POINTER(P)],
            "batch_init_state": [P],
            "batch_step": [P, ctypes.POINTER(StepStats)],
        }
        for name, args in batch.items():
            fn = getattr(lib, "hydro_gpu_" + name)
            fn.argtypes = args
            fn.restype = I
        C = ctypes.c_char_p
        extra = {
            "hydro_gpu_get_desc": [P, ctypes.POINTER(HydroDesc)],
            "hydro_gpu_get_stream": [P, ctypes.POINTER(P)],
            "hydro_gpu_get_time_step": [P, D],
            "hydro_gpu_heat_create": [P, ctypes.POINTER(HeatDesc)],
            "hydro_gpu_heat_step": [P],
            "hydro_output_open": [P, C, C, ctypes.POINTER(P)],
            "hydro_output_write": [P, ctypes.c_double],
            "hydro_output_flush": [P],
            "hydro_output_close": [P],
            "hydro_vts_write_host": [C, I, ctypes.POINTER(I), D, D, I, ctypes.POINTER(C),
                                     ctypes.POINTER(I), ctypes.POINTER(D)],
            "hydro_scalar_output_open": [P, C, ctypes.POINTER(P)],
            "hydro_scalar_output_write": [P, ctypes.c_double, I],
            "hydro_scalar_output_close": [P],
            # learned pressure guess (include/hydro_net.h)
            "hydro_net_create": [I, I, I, I, ctypes.c_ulonglong, ctypes.POINTER(P)],
            "hydro_net_destroy": [P],
            "hydro_net_num_params": [P, ctypes.POINTER(ctypes.c_size_t)],
            "hydro_net_get_params": [P, ctypes.POINTER(ctypes.c_float), ctypes.c_size_t],
            "hydro_net_set_params": [P, ctypes.POINTER(ctypes.c_float), ctypes.c_size_t],
            "hydro_net_pack_sample": [P, P, P, P, ctypes.c_double, P, P],
            "hydro_net_train_step": [P, ctypes.POINTER(P), I, ctypes.c_double, D, P],
            "hydro_net_gradient": [P, ctypes.POINTER(P), I, ctypes.POINTER(ctypes.c_float),
                                   ctypes.c_size_t, D, P],
            "hydro_net_eval_loss": [P, ctypes.POINTER(P), I, D, P],
            "hydro_net_predict": [P, P, P, ctypes.c_double, P, P],
            "hydro_net_last_predict": [P, D, ctypes.POINTER(I)],
            "hydro_gpu_set_pressure_guess": [P, P, I, ctypes.c_double],
            "hydro_gpu_get_guess_stats": [P, ctypes.POINTER(ctypes.c_longlong),
                                          ctypes.POINTER(ctypes.c_longlong),
                                          ctypes.POINTER(ctypes.c_longlong)],
            "hydro_conv3d_forward": [I, I, I, I, I, I, P, P, P, P, I, P, P],
            "hydro_conv3d_backward_data": [I, I, I, I, I, I, P, P, P, P, P, P],
            "hydro_conv3d_backward_weight": [I, I, I, I, I, I, P, P, P, P, P],
        }
        for name, args in extra.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = I
        lib.hydro_net_sample_bytes.argtypes = [P]
        lib.hydro_net_sample_bytes.restype = ctypes.c_size_t
    else:
        stencil.argtypes = [I, I, I, I, D, ctypes.c_double, ctypes.c_long,
                            ctypes.c_double, D, D, I, ctypes.c_double, I,
                            ctypes.POINTER(I), D]
    stencil.restype = I


def fluid_mask(d):
    """Cells outside the rigid box (centre not in [rigid_box_lo,
    rigid_box_hi], inclusive), or None when the case has no box."""
    if not d.rigid_box:
        return None
    import numpy as np
    n = [d.n[k] if k < d.dim else 1 for k in range(3)]
    idx = np.arange(n[0] * n[1] * n[2])
    mi = [idx % n[0], (idx // n[0]) % n[1], idx // (n[0] * n[1])]
    inside = np.ones(idx.size, dtype=bool)
    for k in range(d.dim):
        h = (d.hi[k] - d.lo[k]) / d.n[k]
        xc = d.lo[k] + (mi[k] + 0.5) * h
        inside &= (d.rigid_box_lo[k] <= xc) & (xc <= d.rigid_box_hi[k])
    return ~inside


def desc_to_dict(d):
    """Plain-dict form of a HydroDesc (fixtures, logs)."""
    out = {}
    for name, ctype in HydroDesc._fields_:
        if name == "stream":
            continue
        v = getattr(d, name)
        if hasattr(v, "__len__"):
            v = [list(x) if hasattr(x, "__len__") else x for x in v]
        out[name] = v
    return out


def desc_from_dict(src):
    d = default_desc()
    for name, ctype in HydroDesc._fields_:
        if name == "stream" or name not in src:
            continue
        v = src[name]
        if isinstance(v, list):
            arr = getattr(d, name)
            for i, x in enumerate(v):
                if isinstance(x, list):
                    for j, y in enumerate(x):
                        arr[i][j] = y
                else:
                    arr[i] = x
        else:
            setattr(d, name, v)
    return d
