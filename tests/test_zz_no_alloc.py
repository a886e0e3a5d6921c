"""The no-allocation distance-driven projector (sgb_bdd_project_noalloc), called through
the C ABI.

Some callers cannot let a library call cudaMalloc: services that keep their device
memory fixed after start-up, and hosts whose device memory belongs to another allocator.
For them the library keeps the projector's scratch in an array of its own.  This test
checks, on two calls in a row with different geometries (the second call reuses the
scratch the first one left behind), that the result equals the allocating entry point
sgb_bdd_project within the parity tolerance of the other GPU tests, that the calls make no
device allocation (the library's own allocation counter, sgb_device_alloc_count, does not
move across them), and that a request larger than the array is refused with a clear error.  It is collected last so a failing
run that stops at the first failure has already run every other test.
"""
import ctypes
import math

import numpy as np
import pytest

from sinograms import _lib

pytestmark = pytest.mark.gpu

RTOL_RMSE = 1e-5  # as tests/test_gpu_parity.py
MAX_REL = 1e-4


def _geoms():
    # (DSD, DS0, pSize, dSize, nPix, nDet, na): a reduced test/sys2/bdd_2d.jl geometry and a
    # second, larger one, so the second call overwrites different scratch extents
    return [(949.0, 541.0, 4.0, 4.0956, 128, 226, 90), (600.0, 380.0, 1.5, 1.7, 96, 160, 121)]


def _call(fn, phantom, sino, g, angle, stream):
    DSD, DS0, pSize, dSize, nPix, nDet, na = g
    return fn(ctypes.c_void_p(phantom.data_ptr()), nPix, nDet, na, ctypes.c_void_p(angle.ctypes.data), DSD, DS0,
              pSize, dSize, ctypes.c_void_p(sino.data_ptr()), stream)


def test_bdd_project_noalloc_matches_allocating_entry_point(cuda):
    import torch
    L = _lib.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call, g in enumerate(_geoms()):
        DSD, DS0, pSize, dSize, nPix, nDet, na = g
        angle = np.ascontiguousarray(np.arange(na) * (2 * math.pi / na), dtype=np.float64)
        rng = np.random.default_rng(100 + call)
        phantom = torch.as_tensor(rng.random((nPix, nPix), dtype=np.float32), device="cuda")
        out = torch.full((nDet, na), float("nan"), device="cuda")  # must be fully overwritten
        allocs = L.sgb_device_alloc_count()
        assert _call(L.sgb_bdd_project_noalloc, phantom, out, g, angle, stream) == _lib.SGB_OK, _lib.last_error()
        torch.cuda.synchronize()
        assert L.sgb_device_alloc_count() == allocs, "the no-allocation entry point allocated device memory"
        ref = torch.empty((nDet, na), device="cuda")
        st = L.sgb_bdd_project(ctypes.c_void_p(phantom.data_ptr()), nPix, nDet, na,
                               ctypes.c_void_p(angle.ctypes.data), DSD, DS0, pSize, dSize,
                               ctypes.c_void_p(ref.data_ptr()), _lib.SGB_DEVICE_PTRS, stream)
        assert st == _lib.SGB_OK, _lib.last_error()
        torch.cuda.synchronize()
        o, r = out.cpu().numpy().astype(np.float64), ref.cpu().numpy().astype(np.float64)
        assert np.isfinite(o).all()
        rmse = np.linalg.norm(o - r) / np.linalg.norm(r)
        assert rmse <= RTOL_RMSE and np.abs(o - r).max() <= MAX_REL * np.abs(r).max(), (call, rmse)


def test_bdd_project_noalloc_rejects_oversized_requests(cuda):
    import torch
    L = _lib.lib()
    na, nDet, nPix = 2048, 4096, 64  # per-view tables of ~134 MB exceed the 16 MiB array
    angle = np.zeros(na)
    phantom = torch.zeros((nPix, nPix), device="cuda")
    out = torch.zeros((nDet, na), device="cuda")
    st = L.sgb_bdd_project_noalloc(ctypes.c_void_p(phantom.data_ptr()), nPix, nDet, na,
                                   ctypes.c_void_p(angle.ctypes.data), 900.0, 500.0, 1.0, 1.0,
                                   ctypes.c_void_p(out.data_ptr()), None)
    assert st == _lib.SGB_ERR_ARG
    assert "scratch" in _lib.last_error()
