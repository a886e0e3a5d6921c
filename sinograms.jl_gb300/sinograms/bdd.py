"""Branchless distance-driven projector pair, src/sys2/bdd_2d.jl, on the GPU.

``geo`` is the reference's named tuple: DSD, DS0, pSize, dSize, nPix, nDet, angle.
Layouts follow the reference: the phantom is Julia (nPix, nPix) with row = y (row 1 at
the top) and col = x, i.e. numpy ``phantom_np[col, row]``; the sinogram is Julia
(na, nDet), i.e. numpy ``(nDet, na)``.

Extension: ``BddGeo.arc = True`` (or an ``arc`` key in a dict geo) puts the detector boundaries
on the arc of radius DSD about the source, for SinoFanArc scans; the reference's pair is
flat-only (bdd_2d.jl:28-29).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._arrays import Arr, empty, f64, flags_for, out_buffer, plan_call, ptr, stream_for
from .filters import SinogramsArgumentError
from .geom import _ar, _dso


@dataclass
class BddGeo:
    DSD: float
    DS0: float
    pSize: float
    dSize: float
    nPix: int
    nDet: int
    angle: np.ndarray
    arc: bool = False

    @classmethod
    def from_geoms(cls, rg, ig):
        """geo tuple as built in test/sys2/bdd_2d.jl:21-22 from a fan-beam SinoGeom + ImageGeom;
        a SinoFanArc gives the arc-detector pair."""
        return cls(rg.dsd, _dso(rg), ig.deltas[0], rg.d, ig.dims[0], rg.nb, _ar(rg), bool(getattr(rg, "kind", "") == "arc"))


def _g(geo, k):
    if k == "arc":
        return bool(geo.get("arc", False)) if isinstance(geo, dict) else bool(getattr(geo, "arc", False))
    return geo[k] if isinstance(geo, dict) else getattr(geo, k)


def _run(fn, x, geo, out_shape):
    a = Arr(x)
    ang = f64(_g(geo, "angle"))
    out = empty(out_shape, a)
    flags = flags_for(a.device) | (_lib.SGB_BDD_ARC if _g(geo, "arc") else 0)
    st = getattr(_lib.lib(), fn)(a.ptr, int(_g(geo, "nPix")), int(_g(geo, "nDet")), len(ang), ptr(ang),
                                 float(_g(geo, "DSD")), float(_g(geo, "DS0")), float(_g(geo, "pSize")),
                                 float(_g(geo, "dSize")), ptr(out), flags, stream_for(a.device))
    if st == _lib.SGB_ERR_ARG:
        raise SinogramsArgumentError(_lib.last_error())
    _lib.check(st, fn)
    return out


def project_bdd(phantom, geo):
    """sinogram = project_bdd(phantom, geo), bdd_2d.jl:17-110 (numpy (nDet, na) out)."""
    n = int(_g(geo, "nPix"))
    if tuple(Arr(phantom).shape) != (n, n):
        raise SinogramsArgumentError("phantom must be (nPix, nPix)")
    return _run("sgb_bdd_project", phantom, geo, (int(_g(geo, "nDet")), len(_g(geo, "angle"))))


def backproject_bdd(sinogram, geo):
    """image = backproject_bdd(sinogram, geo), bdd_2d.jl:119-220 (numpy (nPix, nPix))."""
    n = int(_g(geo, "nPix"))
    return _run("sgb_bdd_backproject", sinogram, geo, (n, n))


class BddPlan:
    """The projector pair for one geo tuple with its geometry kept on the GPU
    (sgb_bdd_plan): project / backproject give the results of project_bdd /
    backproject_bdd.  CUDA tensors stay on the device; with sync=False a call only
    enqueues its work on torch's current stream.  Calls on one plan share its scratch:
    keep them on one stream."""

    def __init__(self, geo):
        self.geo = geo
        self.nPix, self.nDet = int(_g(geo, "nPix")), int(_g(geo, "nDet"))
        ang = f64(_g(geo, "angle"))
        self.na = len(ang)
        self._h = ctypes.c_void_p()
        det = _lib.SGB_ARC if _g(geo, "arc") else _lib.SGB_FLAT
        st = _lib.lib().sgb_bdd_plan_create_det(self.nPix, self.nDet, self.na, ptr(ang), float(_g(geo, "DSD")),
                                                float(_g(geo, "DS0")), float(_g(geo, "pSize")),
                                                float(_g(geo, "dSize")), det, ctypes.byref(self._h))
        if st == _lib.SGB_ERR_ARG:
            raise SinogramsArgumentError(_lib.last_error())
        _lib.check(st, "bdd_plan_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib._lib is not None:
            _lib.lib().sgb_bdd_plan_destroy(h)
            self._h = None

    def _call(self, fn, x, out_shape, out, sync):
        a = Arr(x)
        y = out_buffer(out, out_shape, a)
        flags, st = plan_call(a.device, sync)
        _lib.check(getattr(_lib.lib(), fn)(self._h, a.ptr, ptr(y), flags, st), fn)
        return y

    def project(self, phantom, out=None, sync: bool = True):
        """project_bdd(phantom, geo): (nPix, nPix) -> (nDet, na)."""
        if tuple(Arr(phantom).shape) != (self.nPix, self.nPix):
            raise SinogramsArgumentError("phantom must be (nPix, nPix)")
        return self._call("sgb_bdd_plan_project", phantom, (self.nDet, self.na), out, sync)

    def backproject(self, sinogram, out=None, sync: bool = True):
        """backproject_bdd(sinogram, geo): (nDet, na) -> (nPix, nPix)."""
        if tuple(Arr(sinogram).shape) != (self.nDet, self.na):
            raise SinogramsArgumentError("sinogram must be (nDet, na)")
        return self._call("sgb_bdd_plan_backproject", sinogram, (self.nPix, self.nPix), out, sync)
