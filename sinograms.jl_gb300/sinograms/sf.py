"""Separable-footprint (SF-TR) projector pair for 2D parallel and fan beams, and _tau.

The reference sizes this system model's footprints (``footprint_size``, src/sys2/footprint.jl:19-36)
and documents ``_tau`` (src/geom/tau.jl:7-60) as the "footprint center and support", but it has no
projector for it.  This pair is the SF-TR model of Long, Fessler & Balter (IEEE Trans. Med. Imag.
29(11), 2010) in 2D: each pixel's footprint is the trapezoid through the projections of its four
corners, scaled by its chord along the ray through its centre, and a sinogram sample is the
footprints' integral over the detector bin (a bin-averaged line integral; exact for parallel beams).
Both directions run on the GPU (libsinogb300.so); ``backproject`` is the adjoint of ``project``.

Layouts follow this package's numpy order: an image (nx, ny) is numpy ``(ny, nx)`` and a sinogram
(nb, na) is numpy ``(na, nb)``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._arrays import Arr, empty, f64, flags_for, out_buffer, plan_call, ptr, stream_for
from .filters import SinogramsArgumentError
from .geom import ImageGeom, c_struct, is_ct


def _tau(rg, x, y) -> np.ndarray:
    """_tau(rg, x, y), tau.jl:7-60: projected s/ds of the points (x, y) in every view, numpy
    (na, n) (the reference's n x na matrix)."""
    if is_ct(rg):
        raise SinogramsArgumentError("_tau here takes a 2D SinoGeom")
    x, y = f64(np.ravel(x)), f64(np.ravel(y))
    if x.shape != y.shape:
        raise SinogramsArgumentError("x,y axes")  # tau.jl:44
    out = np.zeros((int(rg.na), len(x)))
    _lib.check(_lib.lib().sgb_tau_sino(ctypes.byref(c_struct(rg)), ptr(x), ptr(y), len(x), ptr(out)), "tau")
    return out


def _check(st: int, what: str) -> None:
    if st == _lib.SGB_ERR_ARG:
        raise SinogramsArgumentError(_lib.last_error())
    _lib.check(st, what)


class SFPlan:
    """The SF pair for one SinoGeom (SinoPar, SinoFanArc, SinoFanFlat) and 2D ImageGeom, with its
    per-view constants and boundary-ray table kept on the GPU.  CUDA tensors stay on the device;
    with sync=False a call only enqueues its work on torch's current stream.  Calls on one plan share
    its staging buffers: keep them on one stream."""

    def __init__(self, rg, ig: ImageGeom):
        if is_ct(rg) or getattr(rg, "kind", None) not in ("par", "arc", "flat"):
            raise SinogramsArgumentError("SFPlan needs a SinoPar, SinoFanArc or SinoFanFlat")
        if ig.ndim != 2:
            raise SinogramsArgumentError("SFPlan needs a 2D ImageGeom")
        self.rg, self.ig = rg, ig
        self.nx, self.ny = ig.dims
        self.nb, self.na = int(rg.nb), int(rg.na)
        self._h = ctypes.c_void_p()
        _check(_lib.lib().sgb_sf_plan_create(ctypes.byref(c_struct(rg)), ctypes.byref(ig.c_struct()),
                                             ctypes.byref(self._h)), "sf_plan_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib._lib is not None:
            _lib.lib().sgb_sf_plan_destroy(h)
            self._h = None

    @property
    def line_splits(self) -> int:
        """Thread blocks the forward projector splits each (view, bin chunk)'s image lines over."""
        v = ctypes.c_int()
        _check(_lib.lib().sgb_sf_plan_get_line_splits(self._h, ctypes.byref(v)), "sf_plan_get_line_splits")
        return v.value

    @line_splits.setter
    def line_splits(self, n: int) -> None:
        _check(_lib.lib().sgb_sf_plan_set_line_splits(self._h, int(n)), "sf_plan_set_line_splits")

    def _call(self, fn, x, in_shape, out_shape, out, sync):
        a = Arr(x)
        if tuple(a.shape) != in_shape:
            raise SinogramsArgumentError(f"input must have numpy shape {in_shape}, got {tuple(a.shape)}")
        y = out_buffer(out, out_shape, a)
        flags, st = plan_call(a.device, sync)
        _check(getattr(_lib.lib(), fn)(self._h, a.ptr, ptr(y), flags, st), fn)
        return y

    def project(self, image, out=None, sync: bool = True):
        """image (ny, nx) -> sinogram (na, nb)."""
        return self._call("sgb_sf_plan_project", image, (self.ny, self.nx), (self.na, self.nb), out, sync)

    def backproject(self, sino, out=None, sync: bool = True):
        """sinogram (na, nb) -> image (ny, nx), the adjoint of project."""
        return self._call("sgb_sf_plan_backproject", sino, (self.na, self.nb), (self.ny, self.nx), out, sync)


def _one_shot(fn, rg, ig, x, in_shape, out_shape):
    if is_ct(rg) or ig.ndim != 2:
        raise SinogramsArgumentError("the SF pair takes a 2D SinoGeom and a 2D ImageGeom")
    a = Arr(x)
    if tuple(a.shape) != in_shape:
        raise SinogramsArgumentError(f"input must have numpy shape {in_shape}, got {tuple(a.shape)}")
    y = empty(out_shape, a)
    _check(getattr(_lib.lib(), fn)(ctypes.byref(c_struct(rg)), ctypes.byref(ig.c_struct()), a.ptr, ptr(y),
                                   flags_for(a.device), stream_for(a.device)), fn)
    return y


def project_sf(rg, ig: ImageGeom, image):
    """SF projection of image (ny, nx) -> sinogram (na, nb)."""
    return _one_shot("sgb_sf_project", rg, ig, image, tuple(reversed(ig.dims)), (int(rg.na), int(rg.nb)))


def backproject_sf(rg, ig: ImageGeom, sino):
    """SF back-projection (the adjoint) of sinogram (na, nb) -> image (ny, nx)."""
    return _one_shot("sgb_sf_backproject", rg, ig, sino, (int(rg.na), int(rg.nb)), tuple(reversed(ig.dims)))
