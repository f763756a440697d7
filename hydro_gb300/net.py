"""Python mirror of the learned pressure guess (include/hydro_net.h).

``Net`` holds one network of libhydro_gpu.so: its forward, backward and Adam
kernels run in the library on the tensor cores; this module only marshals
device pointers.  Device buffers for packed samples come from torch (memory
plumbing only).

``snapshot_step`` runs one time step through the public step API (the
sequence of hydro_gpu_step: auto time step, StartStep, SIMPLE iterations,
FinishStep, advection, property update, hydro2d.hpp:1531-1621) and packs
the (f, rho, p') of its first SIMPLE iteration -- the pressure solve the
guess serves -- into a training sample.
"""
import ctypes

import numpy as np

from . import capi


class Net:
    def __init__(self, n, batch=1, seed=0):
        self.lib = capi.load()
        self.n = tuple(int(v) for v in n)
        self.batch = batch
        self.ptr = ctypes.c_void_p()
        st = self.lib.hydro_net_create(self.n[0], self.n[1], self.n[2], batch, seed,
                                       ctypes.byref(self.ptr))
        if st != capi.OK:
            raise capi.HydroError(st, "hydro_net_create")
        k = ctypes.c_size_t()
        self._check(self.lib.hydro_net_num_params(self.ptr, ctypes.byref(k)), "num_params")
        self.nparam = k.value
        self.sample_bytes = self.lib.hydro_net_sample_bytes(self.ptr)

    @staticmethod
    def _check(st, where):
        if st != capi.OK:
            raise capi.HydroError(st, "hydro_net_" + where)

    def close(self):
        if getattr(self, "ptr", None):
            self.lib.hydro_net_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        self.close()

    @property
    def cells(self):
        return self.n[0] * self.n[1] * self.n[2]

    def get_params(self):
        a = np.empty(self.nparam, dtype=np.float32)
        self._check(self.lib.hydro_net_get_params(
            self.ptr, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), a.size), "get_params")
        return a

    def set_params(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        self._check(self.lib.hydro_net_set_params(
            self.ptr, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), a.size), "set_params")

    def pack(self, rhs_ptr, rho_ptr, pc_ptr, rho_scale, dst_ptr, stream=None):
        self._check(self.lib.hydro_net_pack_sample(self.ptr, rhs_ptr, rho_ptr, pc_ptr, rho_scale,
                                                   dst_ptr, stream), "pack_sample")

    @staticmethod
    def _ptrs(samples):
        arr = (ctypes.c_void_p * len(samples))()
        for i, s in enumerate(samples):
            arr[i] = s if isinstance(s, int) else s.data_ptr()
        return arr

    def train_step(self, samples, lr, stream=None):
        loss = ctypes.c_double()
        self._check(self.lib.hydro_net_train_step(self.ptr, self._ptrs(samples), len(samples),
                                                  lr, ctypes.byref(loss), stream), "train_step")
        return loss.value

    def gradient(self, samples, stream=None):
        g = np.empty(self.nparam, dtype=np.float32)
        loss = ctypes.c_double()
        self._check(self.lib.hydro_net_gradient(
            self.ptr, self._ptrs(samples), len(samples),
            g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), g.size, ctypes.byref(loss),
            stream), "gradient")
        return loss.value, g

    def eval_loss(self, samples, stream=None):
        loss = ctypes.c_double()
        self._check(self.lib.hydro_net_eval_loss(self.ptr, self._ptrs(samples), len(samples),
                                                 ctypes.byref(loss), stream), "eval_loss")
        return loss.value

    def predict(self, rhs_ptr, rho_ptr, rho_scale, out_ptr, stream=None):
        self._check(self.lib.hydro_net_predict(self.ptr, rhs_ptr, rho_ptr, rho_scale, out_ptr,
                                               stream), "predict")

    def last_predict(self):
        ms = ctypes.c_double()
        n = ctypes.c_int()
        self._check(self.lib.hydro_net_last_predict(self.ptr, ctypes.byref(ms), ctypes.byref(n)),
                    "last_predict")
        return ms.value, n.value

    def layer_shapes(self):
        """(cin, cout) of the layers in parameter order (padded channels)."""
        return [(16, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 32), (32, 32),
                (32, 16), (16, 16), (16, 16)]

    def save(self, path):
        np.save(path, self.get_params())

    def load(self, path):
        self.set_params(np.load(path))


def attach(hydro, net, iterations=1, rho_scale=1.0):
    """hydro_gpu_set_pressure_guess: the first `iterations` pressure solves
    of every step of `hydro` (a solver.Hydro) start from the network's guess."""
    st = hydro.lib.hydro_gpu_set_pressure_guess(hydro.ctx, net.ptr if net else None, iterations,
                                                rho_scale)
    if st != capi.OK:
        raise capi.HydroError(st, "hydro_gpu_set_pressure_guess")


def guess_stats(hydro):
    """(kept, dropped, skipped) since the last call (hydro_gpu_get_guess_stats)."""
    used, dropped, skipped = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
    st = hydro.lib.hydro_gpu_get_guess_stats(hydro.ctx, ctypes.byref(used), ctypes.byref(dropped),
                                             ctypes.byref(skipped))
    if st != capi.OK:
        raise capi.HydroError(st, "hydro_gpu_get_guess_stats")
    return used.value, dropped.value, skipped.value


def snapshot_step(hydro, net, rho_scale, dst_ptr):
    """One time step of `hydro` through the public API, packing the first
    SIMPLE iteration's pressure system (f, rho, p') into dst_ptr (device,
    net.sample_bytes).  Returns the step's SIMPLE iteration count."""
    d = hydro.desc
    if d.dt_auto:
        dtm = hydro.auto_time_step()
        dt, dta = dtm * d.cfl, dtm * d.cfl_advection
        if d.dt_max > 0 and dt > d.dt_max:
            dta *= d.dt_max / dt
            dt = d.dt_max
        hydro.set_time_step(dt, dta)
    hydro.start_step()
    it = 0
    while not hydro.is_converged():
        hydro.make_iteration()
        if it == 0:
            net.pack(hydro.field_ptr(capi.F_PRESSURE_RHS), hydro.field_ptr(capi.F_DENSITY),
                     hydro.field_ptr(capi.F_PRESSURE_CORRECTION), rho_scale, dst_ptr,
                     hydro.stream_ptr())
        it += 1
    hydro.finish_step()
    if d.advection_enable:
        hydro.advection_step()
    hydro.update_properties()
    return it
