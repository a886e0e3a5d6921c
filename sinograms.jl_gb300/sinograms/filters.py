"""Ramp filter, windows and view weights (src/fbp/*.jl, src/fbp3/fdk.jl:21-45,
src/fbp2/sino-weight.jl) -- thin wrappers over the library's FP64 plan-time code and
its GPU row filter."""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._arrays import Arr, empty, f64, flags_for, ptr, stream_for
from .geom import _ar, _ds, c_struct, is_ct


class SinogramsArgumentError(ValueError):
    """Raised where the reference throws a String or ErrorException for bad arguments."""


def _call(name, *args):
    st = getattr(_lib.lib(), name)(*args)
    if st == _lib.SGB_ERR_ARG or st == _lib.SGB_ERR_GEOM:
        raise SinogramsArgumentError(_lib.last_error())
    _lib.check(st, name)


# ------------------------------------------------------------------- ramp.jl

def ramp_flat(N: int, ds: float):
    """(h, n) = ramp_flat(N, ds), ramp.jl:86-91."""
    h = np.zeros(N)
    _call("sgb_fbp_ramp", _lib.SGB_FLAT, N, ds, 0.0, ptr(h))
    return h, np.arange(-(N // 2), N // 2)


def ramp_arc(N: int, ds: float, dsd: float):
    """(h, n) = ramp_arc(N, ds, dsd), ramp.jl:67-77."""
    h = np.zeros(N)
    _call("sgb_fbp_ramp", _lib.SGB_ARC, N, ds, dsd, ptr(h))
    return h, np.arange(-(N // 2), N // 2)


def fbp_ramp(rg, N: int, dr: float | None = None):
    """fbp_ramp(rg, N), ramp.jl:24-35; for SinoMoj the keyword ``dr`` (default rg.d) is the ray
    spacing, which varies with the projection angle (ramp.jl:27-30)."""
    if rg.kind == "moj":
        return ramp_flat(N, rg.d if dr is None else dr)
    if dr is not None:
        raise SinogramsArgumentError("dr applies to SinoMoj only")
    if rg.kind == "arc":
        return ramp_arc(N, _ds(rg), rg.dsd)
    return ramp_flat(N, _ds(rg))


# ----------------------------------------------------------------- window.jl

@dataclass(frozen=True)
class Window:
    """Window(shape, cutoff), window.jl:22-31.  shape: "none", "boxcar", "hamming",
    "hann", or a vector (WindowVect)."""
    shape: object = "none"
    cutoff: float = 1.0


def fbp_window(w: Window, N: int) -> np.ndarray:
    """fbp_window(w, N), window.jl:60-74 (fftshift'ed)."""
    out = np.zeros(N)
    if isinstance(w.shape, str):
        _call("sgb_fbp_window", _lib.SGB_WIN[w.shape], float(w.cutoff), N, None, ptr(out))
    else:
        v = f64(w.shape)
        if len(v) != N:
            raise SinogramsArgumentError("N mismatch")  # window.jl:72
        _call("sgb_fbp_window", _lib.SGB_WIN["vect"], float(w.cutoff), N, ptr(v), ptr(out))
    return out


# ----------------------------------------------------------------- filter.jl

def _npad_default(n: int) -> int:
    p = 1
    while p < n + 1:
        p <<= 1
    return p


def fbp_filter(rg, npad: int | None = None, window: Window = Window(), decon1: bool = True) -> np.ndarray:
    """Hk = fbp_filter(rg; npad, window, decon1), filter.jl:32-57."""
    n = rg.ns if is_ct(rg) else rg.nb
    npad = npad or _npad_default(n)
    Hk = np.zeros(npad)
    kind = _lib.SGB_ARC if rg.kind == "arc" else _lib.SGB_FLAT
    if isinstance(window.shape, str):
        _call("sgb_fbp_filter", kind, npad, _ds(rg), getattr(rg, "dsd", 0.0) or 0.0, _lib.SGB_WIN[window.shape],
              float(window.cutoff), None, int(decon1), ptr(Hk))
    else:
        v = f64(window.shape)
        _call("sgb_fbp_filter", kind, npad, _ds(rg), getattr(rg, "dsd", 0.0) or 0.0, _lib.SGB_WIN["vect"],
              float(window.cutoff), ptr(v), int(decon1), ptr(Hk))
    return Hk


def fbp_sino_filter(sino, filter, extra: int = 0):
    """fbp_sino_filter(sino, filter; extra), filter.jl:122-147, on the GPU.

    ``sino`` has nb as its LAST axis (numpy order of Julia's (nb, ...)); the result has
    nb + extra samples per row (the extra ones are zero)."""
    a = Arr(sino)
    nb = a.shape[-1]
    nrows = int(np.prod(a.shape[:-1])) if len(a.shape) > 1 else 1
    Hk = f64(filter)
    out = empty(tuple(a.shape[:-1]) + (nb + extra,), a)
    _call("sgb_fbp_sino_filter", a.ptr, nb, nrows, ptr(Hk), len(Hk), extra, ptr(out), flags_for(a.device),
          stream_for(a.device))
    return out


# ----------------------------------------------------------------- weights

def _angle_weights(ar) -> float:
    """_angle_weights(ar), d-angle.jl:55-65."""
    a = f64(ar)
    w = ctypes.c_double()
    _call("sgb_angle_weight", ptr(a), len(a), ctypes.byref(w))
    return w.value


def parker_weight(rg) -> np.ndarray:
    """parker_weight(rg), parker.jl:58, 111-119, 147-154, returned in numpy order:
    SinoPar (1,1) or (na,1); SinoFan (1,1) or (na,nb); CtFan (1,1,1) or (na,1,ns); SinoMoj
    (1,1) for orbits that are whole multiples of 180 degrees, an error otherwise (parker.jl:122-129)."""
    if rg.kind == "moj":
        if math.trunc(rg.orbit / 180) * 180 != abs(rg.orbit):
            raise SinogramsArgumentError(f"No Parker weighting for Mojette geometry with orbit={abs(rg.orbit)}")
        return np.ones((1, 1), dtype=np.float32)
    c = c_struct(rg)
    if is_ct(rg):
        w = np.zeros(rg.ns * rg.na, dtype=np.float32)
        n0, n2 = ctypes.c_int(), ctypes.c_int()
        _call("sgb_parker_weight_ct", ctypes.byref(c), ptr(w), ctypes.byref(n0), ctypes.byref(n2))
        if n0.value == 1:
            return np.ones((1, 1, 1), dtype=np.float32)
        return w.reshape(rg.na, 1, rg.ns)
    w = np.zeros(rg.nb * rg.na, dtype=np.float32)
    n0, n1 = ctypes.c_int(), ctypes.c_int()
    _call("sgb_parker_weight_sino", ctypes.byref(c), ptr(w), ctypes.byref(n0), ctypes.byref(n1))
    if n0.value == 1 and n1.value == 1:
        return np.ones((1, 1), dtype=np.float32)
    if n0.value == 1:
        return w[: rg.na].reshape(rg.na, 1)
    return w.reshape(rg.na, rg.nb)


def fdk_weight_cyl(rg) -> np.ndarray:
    """fdk_weight_cyl(rg), fdk.jl:39-45 -> numpy (nt, ns)."""
    w = np.zeros(rg.ns * rg.nt)
    c = c_struct(rg)
    _call("sgb_fdk_weight_cyl", ctypes.byref(c), ptr(w))
    return w.reshape(rg.nt, rg.ns)


def fbp_sino_weight(rg) -> np.ndarray:
    """fbp_sino_weight(rg), sino-weight.jl:12-16 -> (nb,)."""
    w = np.zeros(rg.nb)
    c = c_struct(rg)
    _call("sgb_fbp_sino_weight", ctypes.byref(c), ptr(w))
    return w


def fdk_view_weight(rg) -> np.ndarray:
    """_fdk_weights(rg), plan3.jl:75-80 (numpy (1|na, nt, ns)).  CtPar, which the reference
    does not reconstruct, takes the view weights of the equivalent SinoPar (no cylinder
    weight)."""
    from .geom import CtPar, SinoPar
    if isinstance(rg, CtPar):
        sp = SinoPar(nb=rg.ns, d=rg.ds, offset=rg.offset_s, na=rg.na, orbit=rg.orbit, orbit_start=rg.orbit_start)
        pw = parker_weight(sp)
        return pw.reshape(pw.shape[0], 1, 1) * _angle_weights(_ar(rg))
    return parker_weight(rg) * fdk_weight_cyl(rg)[None] * _angle_weights(_ar(rg))


def fbp_view_weight(rg) -> np.ndarray:
    """_fbp_weights(rg), plan2.jl:141-145."""
    return parker_weight(rg) * _angle_weights(_ar(rg))
