"""ctypes binding of libsinogb300.so (the C ABI in include/sinogb300.h).

The shared library is built in-tree by ``sinograms.jl_gb300/build.py``.  There is no
CPU fallback: if the library is missing, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "libsinogb300.so")

SGB_OK, SGB_ERR_ARG, SGB_ERR_CUDA, SGB_ERR_NOMEM, SGB_ERR_GEOM, SGB_ERR_UNSUPPORTED, SGB_ERR_TIMEOUT = range(7)
SGB_DEVICE_PTRS, SGB_ASYNC, SGB_BDD_ARC = 1, 2, 4
SGB_PAR, SGB_ARC, SGB_FLAT = 0, 1, 2
SGB_WIN = {"none": 0, "boxcar": 1, "hamming": 2, "hann": 3, "vect": 4}
SGB_STORE_F32, SGB_STORE_BF16, SGB_STORE_F16 = 0, 1, 2
SGB_SRC_CIRCLE, SGB_SRC_HELIX = 0, 1

c_int, c_ll, c_double, c_float, c_void_p = ctypes.c_int, ctypes.c_longlong, ctypes.c_double, ctypes.c_float, ctypes.c_void_p
P = c_void_p
PD = ctypes.POINTER(ctypes.c_double)


class SinoGeomC(ctypes.Structure):
    _fields_ = [("kind", c_int), ("nb", c_int), ("d", c_double), ("offset", c_float), ("na", c_int),
                ("orbit", c_double), ("orbit_start", c_double), ("source_offset", c_double),
                ("dsd", c_double), ("dod", c_double)]


class CtGeomC(ctypes.Structure):
    _fields_ = [("kind", c_int), ("ns", c_int), ("nt", c_int), ("ds", c_double), ("dt", c_double),
                ("offset_s", c_float), ("offset_t", c_float), ("na", c_int), ("orbit", c_double),
                ("orbit_start", c_double), ("source_offset", c_double), ("dsd", c_double), ("dod", c_double),
                ("src", c_int), ("pitch", c_float), ("source_z0", c_double)]


class ImageGeomC(ctypes.Structure):
    _fields_ = [("ndim", c_int), ("dims", c_int * 3), ("deltas", c_double * 3), ("offsets", c_double * 3),
                ("mask", P)]


class FilterOptsC(ctypes.Structure):
    _fields_ = [("window_shape", c_int), ("cutoff", c_double), ("window_vect", P), ("npad", c_int),
                ("decon1", c_int), ("filter", P), ("storage", c_int), ("source_z", c_int)]


# (name, restype, argtypes)
_SIGS = {
    "sgb_version": (c_int, []),
    "sgb_last_error": (c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "sgb_launch_count": (c_ll, []),
    "sgb_device_alloc_count": (c_ll, []),
    "sgb_fbp_ramp": (c_int, [c_int, c_int, c_double, c_double, P]),
    "sgb_fbp_window": (c_int, [c_int, c_double, c_int, P, P]),
    "sgb_fbp_filter": (c_int, [c_int, c_int, c_double, c_double, c_int, c_double, P, c_int, P]),
    "sgb_angle_weight": (c_int, [P, c_int, P]),
    "sgb_parker_weight_sino": (c_int, [P, P, P, P]),
    "sgb_parker_weight_ct": (c_int, [P, P, P, P]),
    "sgb_fdk_weight_cyl": (c_int, [P, P]),
    "sgb_source_zs": (c_int, [P, P]),
    "sgb_footprint_size_sino": (c_int, [P, P, P]),
    "sgb_footprint_size_ct": (c_int, [P, P, P]),
    "sgb_zwart_powell": (c_double, [c_double, c_double]),
    "sgb_zwart_powell_sino": (c_int, [P, c_int, P, c_int, P, c_int, P]),
    "sgb_selftest_wait_timeout": (c_int, [c_ll, P]),
    "sgb_tau_sino": (c_int, [P, P, P, c_ll, P]),
    "sgb_sf_plan_create": (c_int, [P, P, P]),
    "sgb_sf_plan_project": (c_int, [P, P, P, c_int, P]),
    "sgb_sf_plan_backproject": (c_int, [P, P, P, c_int, P]),
    "sgb_sf_plan_destroy": (c_int, [P]),
    "sgb_sf_plan_set_line_splits": (c_int, [P, c_int]),
    "sgb_sf_plan_get_line_splits": (c_int, [P, P]),
    "sgb_sf_project": (c_int, [P, P, P, P, c_int, P]),
    "sgb_sf_backproject": (c_int, [P, P, P, P, c_int, P]),
    "sgb_fbp_sino_weight": (c_int, [P, P]),
    "sgb_fbp_sino_filter": (c_int, [P, c_int, c_ll, P, c_int, c_int, P, c_int, P]),
    "sgb_cbct_back": (c_int, [P, P, c_int, c_int, c_int, P, c_double, c_double, c_double, c_double, c_float,
                              c_float, c_int, P, P, P, c_int, c_int, c_int, P, c_int, c_int, P]),
    "sgb_fbp_back_par": (c_int, [P, P, c_int, c_int, P, P, c_double, c_float, P, P, c_int, c_int, P, c_int,
                                 c_int, P]),
    "sgb_fbp_back_fan": (c_int, [P, P, c_int, c_int, P, P, c_double, c_double, c_double, c_int, c_double,
                                 c_float, P, P, c_int, c_int, P, c_int, c_int, P]),
    "sgb_bdd_project": (c_int, [P, c_int, c_int, c_int, P, c_double, c_double, c_double, c_double, P, c_int, P]),
    "sgb_bdd_project_noalloc": (c_int, [P, c_int, c_int, c_int, P, c_double, c_double, c_double, c_double, P,
                                        P]),
    "sgb_bdd_backproject": (c_int, [P, c_int, c_int, c_int, P, c_double, c_double, c_double, c_double, P, c_int,
                                    P]),
    "sgb_bdd_plan_create": (c_int, [c_int, c_int, c_int, P, c_double, c_double, c_double, c_double, P]),
    "sgb_bdd_plan_create_det": (c_int, [c_int, c_int, c_int, P, c_double, c_double, c_double, c_double, c_int,
                                        P]),
    "sgb_bdd_plan_project": (c_int, [P, P, P, c_int, P]),
    "sgb_bdd_plan_backproject": (c_int, [P, P, P, c_int, P]),
    "sgb_bdd_plan_destroy": (c_int, [P]),
    "sgb_ellipse_sino": (c_int, [P, P, c_int, P, c_int, P]),
    "sgb_ellipsoid_proj": (c_int, [P, P, c_int, P, c_int, P]),
    "sgb_ellipse_image": (c_int, [P, P, c_int, c_int, P, c_int, P]),
    "sgb_fbp_filter_rows": (c_int, [P, P, P, c_int, c_int, P]),
    "sgb_fbp_backproject": (c_int, [P, P, P, c_int, c_int, P]),
    "sgb_plan_fbp_ct": (c_int, [P, P, P, P]),
    "sgb_plan_fbp_sino": (c_int, [P, P, P, P]),
    "sgb_plan_filter": (c_int, [P, P, P]),
    "sgb_fdk": (c_int, [P, P, P, c_int, P]),
    "sgb_fbp": (c_int, [P, P, P, c_int, c_int, P]),
    "sgb_plan_destroy": (c_int, [P]),
    "sgb_plan_set_timing": (c_int, [P, c_int]),
    "sgb_plan_last_timing": (c_int, [P, P, c_int]),
    "sgb_plan_info": (c_int, [P, P, c_int]),
    "sgb_plan_sync": (c_int, [P, P]),
    "sgb_plan_set_view_passes": (c_int, [P, c_int]),
    "sgb_measure_peaks": (c_int, [P, c_int, P]),
    "sgb_lf_create": (c_int, [c_float, P, ctypes.c_ulonglong, P]),
    "sgb_lf_num_params": (c_int, [P]),
    "sgb_lf_get_params": (c_int, [P, P, P]),
    "sgb_lf_apply": (c_int, [P, P, c_ll, c_int, P, c_int, P]),
    "sgb_lf_loss_grad": (c_int, [P, P, P, c_ll, c_int, P, P, c_int, P]),
    "sgb_lf_train_step": (c_int, [P, P, P, c_ll, c_int, c_float, P, c_int, P]),
    "sgb_lf_get_state": (c_int, [P, P, P, P]),
    "sgb_lf_set_state": (c_int, [P, P, P, c_ll]),
    "sgb_lf_destroy": (c_int, [P]),
    "sgb_batch_fdk_create": (c_int, [c_int, P, P, P, P]),
    "sgb_batch_fdk_set_input": (c_int, [P, c_int, P, c_int, P]),
    "sgb_batch_fdk_get_output": (c_int, [P, c_int, P, c_int, P]),
    "sgb_batch_fdk_buffers": (c_int, [P, c_int, P, P]),
    "sgb_batch_fdk_run": (c_int, [P, c_int, P]),
    "sgb_batch_fdk_info": (c_int, [P, P, P, c_int]),
    "sgb_batch_fdk_timing": (c_int, [P, P, c_int]),
    "sgb_batch_fdk_destroy": (c_int, [P]),
}

_lib = None


class SinogramsError(RuntimeError):
    """A failed library call (the reference raises a String or ErrorException)."""

    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with sinograms.jl_gb300/build.py "
                               "(the CUDA library is required; there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(2048)
    lib().sgb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int, what: str = "") -> None:
    if status != SGB_OK:
        raise SinogramsError(status, f"{what}: {last_error()} (status {status})")


def launch_count() -> int:
    return int(lib().sgb_launch_count())


def device_alloc_count() -> int:
    """Device allocations (cudaMalloc) the library has made since it was loaded."""
    return int(lib().sgb_device_alloc_count())


def measure_peaks(stream=None) -> dict:
    """On-chip peaks measured on the GPU: shared-memory load bandwidth (bytes/s) and FP32 FMA
    throughput (flop/s)."""
    out = (ctypes.c_double * 2)()
    check(lib().sgb_measure_peaks(out, 2, stream), "measure_peaks")
    return {"smem_load_bytes_per_s": float(out[0]), "fp32_flops_per_s": float(out[1])}


def exported_symbols() -> list[str]:
    return list(_SIGS)
