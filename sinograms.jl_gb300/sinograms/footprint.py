"""sys2 helpers of the reference: footprint_size (src/sys2/footprint.jl) and the
Zwart-Powell box-spline Radon transform (src/sys2/zwart_powell.jl)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._arrays import f64
from .geom import ImageGeom, c_struct, is_ct


def footprint_size(rg, ig: ImageGeom) -> float:
    """footprint_size(st, ig), footprint.jl:19-36: maximum footprint of a pixel in
    detector samples (Float32).  Fans raise SinogramsError("bad dso") when the image's
    radial FOV exceeds 0.99 dso."""
    out = ctypes.c_float()
    fn = "sgb_footprint_size_ct" if is_ct(rg) else "sgb_footprint_size_sino"
    _lib.check(getattr(_lib.lib(), fn)(ctypes.byref(c_struct(rg)), ctypes.byref(ig.c_struct()), ctypes.byref(out)),
               "footprint_size")
    return out.value


def zwart_powell(r, phi):
    """zwart_powell(r, phi), zwart_powell.jl:17-20: Radon transform of the Zwart-Powell box
    spline at radius r (pixel units) and angle phi, elementwise (host, FP64)."""
    f = np.vectorize(lambda a, b: _lib.lib().sgb_zwart_powell(float(a), float(b)), otypes=[np.float64])
    out = f(r, phi)
    return float(out) if np.ndim(out) == 0 else out


def zwart_powell_sino(r, phi, device: bool = False):
    """The grid zwart_powell.(r, phi') of the reference's test (nr x nphi, numpy order
    (nphi, nr)) evaluated on the GPU in FP64."""
    r, phi = f64(r).ravel(), f64(phi).ravel()
    if device:
        import torch
        rd = torch.as_tensor(r, device="cuda")
        pd = torch.as_tensor(phi, device="cuda")
        out = torch.empty((phi.size, r.size), dtype=torch.float64, device="cuda")
        st = _lib.lib().sgb_zwart_powell_sino(ctypes.c_void_p(rd.data_ptr()), r.size, ctypes.c_void_p(pd.data_ptr()),
                                              phi.size, ctypes.c_void_p(out.data_ptr()), _lib.SGB_DEVICE_PTRS,
                                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    else:
        out = np.empty((phi.size, r.size))
        st = _lib.lib().sgb_zwart_powell_sino(r.ctypes.data, r.size, phi.ctypes.data, phi.size, out.ctypes.data, 0,
                                              None)
    _lib.check(st, "zwart_powell_sino")
    return out
