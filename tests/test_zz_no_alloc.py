"""hydro_gpu_stencil_solve_noalloc against hydro_gpu_stencil_solve.

The no-allocation entry point exists for callers that may not call
cudaMalloc -- a plugin inside a host application that owns all device
memory, or a latency-critical loop that cannot afford cudaMalloc's possible
device synchronisation or out-of-memory failure.  It solves the same rows
as hydro_gpu_stencil_solve but takes its scratch from a fixed device array
of the library instead of a caller workspace.

Two calls in a row on each of two systems (a 2D singular system, then a 3D
system with a pinned cell), each through the C-ABI, must give the existing
entry point's answer within the tolerance of the other stencil-solve tests;
the second call of each must leave the device's free memory unchanged.  This file is named
so that pytest collects it last; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from hydro_gb300 import capi

pytestmark = pytest.mark.gpu


def _system(rng, dim, n, pinned):
    d = capi.default_desc()
    d.dim = dim
    for k in range(3):
        d.n[k] = n[k]
    kf = rng.uniform(0.5, 2.0, d.nfaces)
    c = rng.normal(size=d.ncells)
    if pinned < 0:
        c -= c.mean()
    return d.ncells, kf, c


def test_noalloc_matches_workspace_solve_twice(built):
    import torch
    lib = capi.load()
    dev = torch.device("cuda")
    rng = np.random.default_rng(11)
    cases = [(2, (40, 24, 1), -1, 0.0), (3, (12, 10, 9), 57, 0.25)]
    for dim, n, pin, pval in cases:
        nc, kf, c = _system(rng, dim, n, pin)
        nz = n[2] if dim == 3 else 1
        dk = torch.from_numpy(kf).to(dev)
        dc = torch.from_numpy(c).to(dev)
        x_ref = torch.zeros(nc, dtype=torch.float64, device=dev)
        x_new = torch.zeros(nc, dtype=torch.float64, device=dev)
        ws = torch.empty(lib.hydro_gpu_stencil_workspace_size(dim, n[0], n[1], nz),
                         dtype=torch.uint8, device=dev)
        torch.cuda.synchronize()
        it_a, res_a = ctypes.c_int(), ctypes.c_double()
        st_a = lib.hydro_gpu_stencil_solve(dim, n[0], n[1], nz, dk.data_ptr(), 0.0, pin, pval,
                                           dc.data_ptr(), x_ref.data_ptr(), 0, 1e-12, 5000,
                                           ws.data_ptr(), None, ctypes.byref(it_a),
                                           ctypes.byref(res_a))
        a = x_ref.cpu().numpy()
        assert st_a == capi.OK, st_a
        for call in range(2):
            # the second call of a case (every kernel it launches already
            # loaded) must leave the device's free memory and torch's
            # allocations unchanged: the entry point allocates nothing
            x_new.fill_(0.0)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            held0 = torch.cuda.memory_allocated()
            it_b, res_b = ctypes.c_int(), ctypes.c_double()
            st_b = lib.hydro_gpu_stencil_solve_noalloc(dim, n[0], n[1], nz, dk.data_ptr(), 0.0,
                                                       pin, pval, dc.data_ptr(), x_new.data_ptr(),
                                                       0, 1e-12, 5000, None, ctypes.byref(it_b),
                                                       ctypes.byref(res_b))
            torch.cuda.synchronize()
            if call == 1:
                assert torch.cuda.mem_get_info()[0] == free0
                assert torch.cuda.memory_allocated() == held0
            assert st_b == capi.OK, st_b
            b = x_new.cpu().numpy()
            rel = np.linalg.norm(b - a) / np.linalg.norm(a)
            assert rel <= 1e-9, (dim, n, call, rel)
            assert res_b.value <= 1e-12 and it_b.value == it_a.value


def test_noalloc_rejects_oversize(built):
    lib = capi.load()
    it, res = ctypes.c_int(), ctypes.c_double()
    # 80^3 = 512000 cells > HYDRO_NOALLOC_MAX_CELLS: rejected before any GPU work
    st = lib.hydro_gpu_stencil_solve_noalloc(3, 80, 80, 80, None, 0.0, -1, 0.0, None, None, 0,
                                             1e-8, 10, None, ctypes.byref(it), ctypes.byref(res))
    assert st == capi.ERR_ARG
