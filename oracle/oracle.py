"""CPU oracle for the Sinograms.jl reconstruction hot path (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import this module; the product (``libsinogb300.so`` and the ``sinograms`` python mirror)
never does.  The arithmetic lives in ``oracle.c`` (double-precision build
``liboracle64.so``, float build ``liboracle32.so``); this file restates the reference's
plan-level orchestration and geometry scalars on top of it.

Array convention: numpy C-order with the Julia dimensions reversed, so memory is
identical to the reference's column-major arrays.  proj (ns,nt,na) is numpy
``(na, nt, ns)``; sino (nb,na) is ``(na, nb)``; image (nx,ny[,nz]) is ``([nz,] ny, nx)``.

Geometry objects are read by attribute or by key (duck typing); fields follow the
reference structs (src/geom/type2.jl:95-159, type3.jl:102-184):
  2D: kind in {"par","arc","flat"}, nb, d, offset, na, orbit, orbit_start,
      source_offset, dsd, dod
  3D: kind in {"arc","flat"}, ns, nt, ds, dt, offset_s, offset_t, na, orbit,
      orbit_start, source_offset, dsd, dod
  image: dims, deltas, offsets, mask (bool array in numpy order, or None)
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS: dict[int, ctypes.CDLL] = {}

_c_int, _c_long, _c_double, _c_float = ctypes.c_int, ctypes.c_long, ctypes.c_double, ctypes.c_float
_P = ctypes.c_void_p


def build() -> None:
    """Compile liboracle64.so / liboracle32.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib(bits: int = 64) -> ctypes.CDLL:
    if bits not in _LIBS:
        path = os.path.join(_HERE, f"liboracle{bits}.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        for name in ("orc_ramp_flat", "orc_ramp_arc", "orc_window", "orc_fbp_filter", "orc_sino_filter",
                     "orc_angle_weight", "orc_parker_par", "orc_parker_fan_short", "orc_cbct_back",
                     "orc_back_par", "orc_back_fan", "orc_bdd_project", "orc_bdd_back", "orc_bdd_project_det",
                     "orc_bdd_back_det", "orc_real_bytes",
                     "orc_num_threads"):
            getattr(L, name).restype = _c_int
        _LIBS[bits] = L
    return _LIBS[bits]


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _f(g, name, default=None):
    if isinstance(g, dict):
        return g.get(name, default)
    return getattr(g, name, default)


def _check(rc, what):
    if rc != 0:
        raise ValueError(f"oracle {what} failed with status {rc}")


# ------------------------------------------------------------------ geometry scalars
# src/geom/common.jl:27-99, sino-geom.jl:18-26, ct-geom.jl:19-23

def ar(g) -> np.ndarray:
    """_ar: angles in radians, common.jl:27-34 + unit.jl:10."""
    na, orbit, start = int(_f(g, "na")), float(_f(g, "orbit")), float(_f(g, "orbit_start", 0.0))
    return (start + np.arange(na) * (orbit / na)) * (math.pi / 180)


def angles_deg(g) -> np.ndarray:
    na, orbit, start = int(_f(g, "na")), float(_f(g, "orbit")), float(_f(g, "orbit_start", 0.0))
    return start + np.arange(na) * (orbit / na)


def is_ct(g) -> bool:
    return _f(g, "ns") is not None


def s_axis(g) -> np.ndarray:
    """_s: sino-geom.jl:18-20 / ct-geom.jl:19-23."""
    if is_ct(g):
        n, d, off = int(_f(g, "ns")), float(_f(g, "ds")), float(np.float32(_f(g, "offset_s", 0.0)))
    else:
        n, d, off = int(_f(g, "nb")), float(_f(g, "d")), float(np.float32(_f(g, "offset", 0.0)))
    return d * (np.arange(n) - ((n - 1) / 2 + off))


def t_axis(g) -> np.ndarray:
    n, d, off = int(_f(g, "nt")), float(_f(g, "dt")), float(np.float32(_f(g, "offset_t", 0.0)))
    return d * (np.arange(n) - ((n - 1) / 2 + off))


def dso(g) -> float:
    return float(_f(g, "dsd", 0.0)) - float(_f(g, "dod", 0.0))


def gamma(g) -> np.ndarray:
    """_gamma, common.jl:93-97."""
    s = s_axis(g)
    return s / float(_f(g, "dsd")) if _f(g, "kind") == "arc" else np.arctan(s / float(_f(g, "dsd")))


def gamma_max(g) -> float:
    return float(np.max(np.abs(gamma(g))))


def orbit_short(g) -> float:
    """_orbit_short, common.jl:40."""
    return 180 + 2 * math.degrees(gamma_max(g))


def rfov(g) -> float:
    """_rfov, common.jl:59-61."""
    if _f(g, "kind") == "par":
        return float(np.max(np.abs(s_axis(g))))
    return dso(g) * math.sin(gamma_max(g))


def image_axes(ig):
    dims, deltas = tuple(_f(ig, "dims")), tuple(_f(ig, "deltas"))
    offs = tuple(_f(ig, "offsets", (0.0,) * len(dims)) or (0.0,) * len(dims))
    return [float(dl) * (np.arange(n) - ((n - 1) / 2 + float(o))) for n, dl, o in zip(dims, deltas, offs)]


def _mask(ig):
    m = _f(ig, "mask")
    if m is None:
        return None
    return np.ascontiguousarray(m, dtype=np.uint8)


# ------------------------------------------------------------ filter / weights

def ramp(g, N: int) -> np.ndarray:
    """fbp_ramp, ramp.jl:24-35."""
    h = np.zeros(N)
    d = float(_f(g, "ds")) if is_ct(g) else float(_f(g, "d"))
    if _f(g, "kind") == "arc":
        _check(lib().orc_ramp_arc(N, _c_double(d), _c_double(float(_f(g, "dsd"))), _ptr(h)), "ramp_arc")
    else:
        _check(lib().orc_ramp_flat(N, _c_double(d), _ptr(h)), "ramp_flat")
    return h


_SHAPES = {"none": 0, "boxcar": 1, "hamming": 2, "hann": 3, "vect": 4}


def window(N: int, shape: str = "none", cutoff: float = 1.0, vect=None) -> np.ndarray:
    out = np.zeros(N)
    v = None if vect is None else np.ascontiguousarray(vect, dtype=np.float64)
    _check(lib().orc_window(_SHAPES[shape], _c_double(cutoff), N, _ptr(v), _ptr(out)), "window")
    return out


def fbp_filter(g, npad: int | None = None, shape: str = "none", cutoff: float = 1.0, vect=None,
               decon1: bool = True) -> np.ndarray:
    """fbp_filter, filter.jl:32-57."""
    n = int(_f(g, "ns")) if is_ct(g) else int(_f(g, "nb"))
    if npad is None:
        npad = 1 << int(math.ceil(math.log2(n + 1)))
    h = ramp(g, npad)
    win = window(npad, shape, cutoff, vect)
    d = float(_f(g, "ds")) if is_ct(g) else float(_f(g, "d"))
    Hk = np.zeros(npad)
    _check(lib().orc_fbp_filter(_ptr(h), npad, _c_double(d), _ptr(win), int(decon1), _ptr(Hk)), "fbp_filter")
    return Hk


def angle_weight(g) -> float:
    a = np.ascontiguousarray(ar(g))
    w = _c_double()
    _check(lib().orc_angle_weight(_ptr(a), len(a), ctypes.byref(w)), "angle_weight")
    return w.value


def parker_weight(g) -> np.ndarray:
    """parker_weight, parker.jl:58, 111-119, 147-154.  numpy-order shapes:
    SinoPar (1,1) or (na,1); SinoFan (1,1) or (na,nb); CtFan (1,1,1) or (na,1,ns)."""
    kind, orbit, na = _f(g, "kind"), float(_f(g, "orbit")), int(_f(g, "na"))
    if kind == "par":
        ad = np.ascontiguousarray(angles_deg(g) - float(_f(g, "orbit_start", 0.0)))
        w = np.zeros(na)
        nw = _c_int()
        _check(lib().orc_parker_par(_c_double(orbit), _ptr(ad), na, _ptr(w), ctypes.byref(nw)), "parker_par")
        return np.ones((1, 1)) if nw.value == 1 else w.reshape(na, 1)
    ct = is_ct(g)
    if math.trunc(orbit / 360) * 360 == orbit:
        return np.ones((1, 1, 1)) if ct else np.ones((1, 1))
    nb = int(_f(g, "ns")) if ct else int(_f(g, "nb"))
    a = np.ascontiguousarray(ar(g))
    gam = np.ascontiguousarray(gamma(g))
    w = np.zeros((na, nb))
    _check(lib().orc_parker_fan_short(nb, na, _ptr(a), _ptr(gam), _c_double(gamma_max(g)), _ptr(w)),
           "parker_fan_short")
    return w.reshape(na, 1, nb) if ct else w


def fdk_weight_cyl(rg) -> np.ndarray:
    """fdk_weight_cyl, fdk.jl:39-45 -> numpy (nt, ns)."""
    s, t = s_axis(rg), t_axis(rg)
    dsd = float(_f(rg, "dsd"))
    S, T = np.meshgrid(s, t)
    if _f(rg, "kind") == "arc":
        return (dso(rg) / dsd) * np.cos(S / dsd) / np.sqrt((T / dsd) ** 2 + 1)
    return dso(rg) / np.sqrt(S ** 2 + T ** 2 + dsd ** 2)


def fdk_weights(rg) -> np.ndarray:
    """_fdk_weights, plan3.jl:75-80.  CtPar (no FBP in the reference): the view weights of
    the equivalent SinoPar, parker_weight_par x dbeta, without a cylinder weight."""
    if _f(rg, "kind") == "par":
        pw = parker_weight(rg)
        return pw.reshape(pw.shape[0], 1, 1) * angle_weight(rg)
    return parker_weight(rg) * fdk_weight_cyl(rg)[None, :, :] * angle_weight(rg)


def fbp_weights(g) -> np.ndarray:
    """_fbp_weights, plan2.jl:141-145."""
    return parker_weight(g) * angle_weight(g)


def fbp_sino_weight(g) -> np.ndarray:
    """fbp_sino_weight, sino-weight.jl:12-16 (nb,)."""
    gam = gamma(g)
    return np.abs(dso(g) * np.cos(gam) - float(_f(g, "source_offset", 0.0)) * np.sin(gam)) / float(_f(g, "dsd"))


def sino_filter(x: np.ndarray, Hk: np.ndarray, extra: int = 0, bits: int = 64) -> np.ndarray:
    """fbp_sino_filter, filter.jl:122-147; x has nb as its LAST numpy axis."""
    dt = np.float64 if bits == 64 else np.float32
    x = np.ascontiguousarray(x, dtype=dt)
    nb = x.shape[-1]
    nrows = x.size // nb
    out = np.zeros(x.shape[:-1] + (nb + extra,), dtype=dt)
    Hk = np.ascontiguousarray(Hk, dtype=np.float64)
    _check(lib(bits).orc_sino_filter(_ptr(x), nb, _c_long(nrows), _ptr(Hk), len(Hk), extra, _ptr(out)),
           "sino_filter")
    return out


# ------------------------------------------------------------------ back-projectors

def source_zs(rg) -> np.ndarray:
    """_source_zs(rg), ct-geom.jl:118-140: zeros for a circle; for a helix (rg["pitch"],
    rg["source_z0"]) z_i = i * pitch * zfov / (na * 360/orbit) + source_z0, zfov = dso/dsd*nt*dt."""
    na = int(_f(rg, "na"))
    if _f(rg, "src", "circle") != "helix":
        return np.zeros(na)
    zfov = dso(rg) / float(_f(rg, "dsd")) * int(_f(rg, "nt")) * float(_f(rg, "dt"))
    pitch = float(np.float32(_f(rg, "pitch", 0.0)))  # CtSourceHelix.pitch::Float32
    dz = 0.0 if na == 1 else pitch * zfov / (na * (360 / float(_f(rg, "orbit"))))
    return np.arange(na) * dz + float(_f(rg, "source_z0", 0.0))


def cbct_back(proj: np.ndarray, rg, ig, ia_skip: int = 1, bits: int = 64, betas=None, zs=None) -> np.ndarray:
    """cbct_back, cbct-back.jl:25-45 -> image numpy (nz, ny, nx).  ``zs`` (per view, length
    units) applies the helical shift t' = mag (z - zs[ia]) the reference leaves commented at
    cbct-back.jl:188; None is the reference's z_src = 0."""
    dt_ = np.float64 if bits == 64 else np.float32
    proj = np.ascontiguousarray(proj, dtype=dt_)
    na, nt, ns = proj.shape
    xc, yc, zc = image_axes(ig)
    nx, ny, nz = len(xc), len(yc), len(zc)
    img = np.zeros((nz, ny, nx), dtype=dt_)
    b = np.ascontiguousarray(ar(rg) if betas is None else betas, dtype=np.float64)
    m = _mask(ig)
    zsd = None if zs is None else np.ascontiguousarray(np.asarray(zs, np.float64) / float(_f(rg, "ds")))
    _check(lib(bits).orc_cbct_back_zs(
        _ptr(img), _ptr(proj), ns, nt, na, _ptr(b), _c_double(float(_f(rg, "dsd", 0.0))), _c_double(dso(rg)),
        _c_double(float(_f(rg, "ds"))), _c_double(float(_f(rg, "dt"))),
        _c_float(float(_f(rg, "offset_s", 0.0))), _c_float(float(_f(rg, "offset_t", 0.0))),
        {"flat": 0, "arc": 1, "par": 2}[_f(rg, "kind")], _ptr(xc), _ptr(yc), _ptr(zc), nx, ny, nz, _ptr(m), ia_skip,
        _ptr(zsd)),
        "cbct_back")
    return img


def fdk(rg, ig, proj: np.ndarray, shape="none", cutoff=1.0, npad=None, decon1=True, bits=64,
        source_z=False) -> np.ndarray:
    """fdk, fdk.jl:65-81 with plan_fbp, plan3.jl:60-72 (source_z: the helical shift of
    cbct_back's commented line 188 with _source_zs(rg))."""
    Hk = fbp_filter(rg, npad, shape, cutoff, decon1=decon1)
    p = np.asarray(proj, dtype=np.float64) * fdk_weights(rg)
    p = sino_filter(p, Hk, bits=bits)
    return cbct_back(p, rg, ig, bits=bits, zs=source_zs(rg) if source_z else None)


def fbp_back(g, ig, sino: np.ndarray, ia_skip: int = 1, bits: int = 64) -> np.ndarray:
    """fbp_back, back-par.jl:184-203 / back-fan.jl:11-32 -> image numpy (ny, nx)."""
    dt_ = np.float64 if bits == 64 else np.float32
    sino = np.ascontiguousarray(sino, dtype=dt_)
    na, nb = sino.shape
    xc, yc = image_axes(ig)
    nx, ny = len(xc), len(yc)
    img = np.zeros((ny, nx), dtype=dt_)
    a = ar(g)[::ia_skip]
    sn, cs = np.ascontiguousarray(np.sin(a)), np.ascontiguousarray(np.cos(a))
    m = _mask(ig)
    if _f(g, "kind") == "par":
        rc = lib(bits).orc_back_par(_ptr(img), _ptr(sino), nb, na, _ptr(sn), _ptr(cs), _c_double(float(_f(g, "d"))),
                                    _c_float(float(_f(g, "offset", 0.0))), _ptr(xc), _ptr(yc), nx, ny, _ptr(m),
                                    ia_skip)
    else:
        rc = lib(bits).orc_back_fan(_ptr(img), _ptr(sino), nb, na, _ptr(sn), _ptr(cs),
                                    _c_double(float(_f(g, "dsd"))), _c_double(dso(g)),
                                    _c_double(float(_f(g, "source_offset", 0.0))), int(_f(g, "kind") == "arc"),
                                    _c_double(float(_f(g, "d"))), _c_float(float(_f(g, "offset", 0.0))),
                                    _ptr(xc), _ptr(yc), nx, ny, _ptr(m), ia_skip)
    _check(rc, "fbp_back")
    return img


def fbp(g, ig, sino: np.ndarray, shape="none", cutoff=1.0, npad=None, decon1=True, bits=64) -> np.ndarray:
    """fbp(plan, sino), fbp.jl:24-38 and :72-86 (2D)."""
    Hk = fbp_filter(g, npad, shape, cutoff, decon1=decon1)
    s = np.asarray(sino, dtype=np.float64)
    if _f(g, "kind") != "par":
        s = s * fbp_sino_weight(g)[None, :]
    s = s * fbp_weights(g)
    s = sino_filter(s, Hk, bits=bits)
    return fbp_back(g, ig, s, bits=bits)


# --------------------------------------------------------------------- bdd_2d.jl

def bdd_geo(DSD, DS0, pSize, dSize, nPix, nDet, angle, arc=False):
    """The reference's geo tuple; arc=True puts the detector boundaries on the arc of radius DSD
    about the source (an extension: the reference pair is flat-only)."""
    return dict(DSD=float(DSD), DS0=float(DS0), pSize=float(pSize), dSize=float(dSize), nPix=int(nPix),
                nDet=int(nDet), angle=np.ascontiguousarray(angle, dtype=np.float64), arc=bool(arc))


def project_bdd(phantom: np.ndarray, geo, bits: int = 64) -> np.ndarray:
    """project_bdd, bdd_2d.jl:17-110.  phantom: Julia (nPix,nPix) [row=y, col=x] as
    numpy (col, row) i.e. ``phantom_np[c, r]``; returns Julia (na,nDet) as numpy (nDet, na)."""
    dt_ = np.float64 if bits == 64 else np.float32
    ph = np.ascontiguousarray(phantom, dtype=dt_)
    na = len(geo["angle"])
    out = np.zeros((geo["nDet"], na), dtype=dt_)
    _check(lib(bits).orc_bdd_project_det(_ptr(ph), geo["nPix"], geo["nDet"], na, _ptr(geo["angle"]),
                                         _c_double(geo["DSD"]), _c_double(geo["DS0"]), _c_double(geo["pSize"]),
                                         _c_double(geo["dSize"]), int(geo.get("arc", False)), _ptr(out)),
           "bdd_project")
    return out


def backproject_bdd(sino: np.ndarray, geo, bits: int = 64) -> np.ndarray:
    """backproject_bdd, bdd_2d.jl:119-220 (numpy layouts as project_bdd)."""
    dt_ = np.float64 if bits == 64 else np.float32
    s = np.ascontiguousarray(sino, dtype=dt_)
    na = len(geo["angle"])
    out = np.zeros((geo["nPix"], geo["nPix"]), dtype=dt_)
    _check(lib(bits).orc_bdd_back_det(_ptr(s), geo["nPix"], geo["nDet"], na, _ptr(geo["angle"]),
                                      _c_double(geo["DSD"]), _c_double(geo["DS0"]), _c_double(geo["pSize"]),
                                      _c_double(geo["dSize"]), int(geo.get("arc", False)), _ptr(out)),
           "bdd_back")
    return out


# ------------------------------------------------------------ analytic phantoms

def ellipse_radon(ell: np.ndarray, r: np.ndarray, phi: np.ndarray) -> np.ndarray:
    ell = np.ascontiguousarray(ell, dtype=np.float64).reshape(-1, 6)
    r, phi = np.broadcast_arrays(np.asarray(r, np.float64), np.asarray(phi, np.float64))
    shape = r.shape
    r, phi = np.ascontiguousarray(r.ravel()), np.ascontiguousarray(phi.ravel())
    out = np.zeros(r.size)
    lib().orc_ellipse_radon(_ptr(ell), len(ell), _ptr(r), _ptr(phi), _c_long(r.size), _ptr(out))
    return out.reshape(shape)


def sino_rays(g):
    """rays(rg) for 2D geometries (sino-geom.jl:99-132) -> (r, phi), numpy (na, nb)."""
    s, b = s_axis(g), ar(g)
    if _f(g, "kind") == "par":
        return np.broadcast_to(s[None, :], (len(b), len(s))), np.broadcast_to(b[:, None], (len(b), len(s)))
    gam = gamma(g)
    r = dso(g) * np.sin(gam)
    return np.broadcast_to(r[None, :], (len(b), len(s))), gam[None, :] + b[:, None]


def ellipse_sino(g, ell) -> np.ndarray:
    r, phi = sino_rays(g)
    return ellipse_radon(ell, r, phi)


def ellipsoid_proj(rg, ell, rows=None) -> np.ndarray:
    """Cone-beam line integrals of ellipsoids, (na, nt, ns).  `rows` (detector row indices)
    limits the work to those rows; the others stay zero."""
    ell = np.ascontiguousarray(ell, dtype=np.float64).reshape(-1, 10)
    s, t, b = (np.ascontiguousarray(v) for v in (s_axis(rg), t_axis(rg), ar(rg)))
    ts = t if rows is None else np.ascontiguousarray(t[np.asarray(rows)])
    part = np.zeros((len(b), len(ts), len(s)))
    lib().orc_ellipsoid_cone(_ptr(ell), len(ell), int(_f(rg, "kind") == "arc"), _ptr(s), len(s), _ptr(ts), len(ts),
                             _ptr(b), len(b), _c_double(dso(rg)), _c_double(float(_f(rg, "dsd"))), _ptr(part))
    if rows is None:
        return part
    out = np.zeros((len(b), len(t), len(s)))
    out[:, np.asarray(rows), :] = part
    return out


def rel_rmse(x, ref) -> float:
    x, ref = np.asarray(x, np.float64), np.asarray(ref, np.float64)
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))


def sino_filter_fft(x: np.ndarray, Hk: np.ndarray, workers: int = 1, chunk_rows: int = 1 << 16) -> np.ndarray:
    """fbp_sino_filter with the reference's own FFT formulation (filter.jl:122-147:
    zero-pad to npad, fft, multiply by Hk, ifft, real part, crop), on the last axis.
    float32 input is transformed in complex64 like FFTW on Float32 data."""
    import scipy.fft as sfft
    npad, nb = len(Hk), x.shape[-1]
    flat = x.reshape(-1, nb)
    out = np.empty_like(flat)
    H = Hk.astype(np.float32 if flat.dtype == np.float32 else np.float64)
    for r0 in range(0, flat.shape[0], chunk_rows):
        blk = flat[r0:r0 + chunk_rows]
        F = sfft.fft(blk, n=npad, axis=-1, workers=workers)
        F *= H
        out[r0:r0 + chunk_rows] = sfft.ifft(F, axis=-1, workers=workers).real[:, :nb]
    return out.reshape(x.shape)


# ---------------------------------------------------------------- sys2
def zwart_powell(r, phi):
    """zwart_powell(r, phi), src/sys2/zwart_powell.jl:17-58 (C restatement, FP64)."""
    f = lib(64).orc_zwart_powell
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_double, ctypes.c_double]
    return np.vectorize(lambda a, b: f(float(a), float(b)))(r, phi)


def zwart_powell_z(r, z):
    """zwart_powell(r, z::NTuple{4}), src/sys2/zwart_powell.jl:23-58: box-spline Radon value for
    direction lengths z (C restatement, FP64)."""
    f = lib(64).orc_zwart_powell_z
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_double] * 5
    z = [float(v) for v in z]
    return np.vectorize(lambda a: f(float(a), *z))(r)


def _kind_code(g) -> int:
    return {"par": 0, "arc": 1, "flat": 2}[_f(g, "kind")]


def tau(g, x, y) -> np.ndarray:
    """_tau(rg, x, y), src/geom/tau.jl:7-60, for a 2D SinoGeom: projected s/ds of the points,
    numpy (na, n) (the reference's n x na matrix)."""
    x = np.ascontiguousarray(np.ravel(x), dtype=np.float64)
    y = np.ascontiguousarray(np.ravel(y), dtype=np.float64)
    b = ar(g)
    out = np.zeros((len(b), len(x)))
    _check(lib(64).orc_tau(_kind_code(g), _ptr(b), len(b), _c_double(float(_f(g, "d"))),
                           _c_double(float(_f(g, "dsd", 0.0))), _c_double(dso(g)),
                           _c_double(float(_f(g, "source_offset", 0.0))), _ptr(x), _ptr(y), _c_long(len(x)),
                           _ptr(out)), "tau")
    return out


def _sf_args(g, ig):
    (nx, ny), (dx, dy) = tuple(_f(ig, "dims"))[:2], tuple(_f(ig, "deltas"))[:2]
    offs = tuple(_f(ig, "offsets", (0.0, 0.0)) or (0.0, 0.0))[:2]
    b = ar(g)
    return b, (_kind_code(g), int(_f(g, "nb")), _c_double(float(_f(g, "d"))),
               _c_double(float(np.float32(_f(g, "offset", 0.0)))), len(b), _ptr(b),
               _c_double(float(_f(g, "dsd", 0.0))), _c_double(dso(g) if _f(g, "kind") != "par" else 0.0),
               _c_double(float(_f(g, "source_offset", 0.0))), int(nx), int(ny), _c_double(float(dx)),
               _c_double(float(dy)), _c_double(float(offs[0])), _c_double(float(offs[1])))


def sf_project(g, ig, image: np.ndarray, bits: int = 64) -> np.ndarray:
    """Separable-footprint (SF-TR) projection of image (numpy (ny, nx)) -> sino (numpy (na, nb));
    the model is stated in oracle.c (orc_sf_project)."""
    dt = np.float64 if bits == 64 else np.float32
    img = np.ascontiguousarray(image, dtype=dt)
    b, args = _sf_args(g, ig)
    out = np.zeros((len(b), int(_f(g, "nb"))), dtype=dt)
    m = _mask(ig)
    _check(lib(bits).orc_sf_project(*args, _ptr(m), _ptr(img), _ptr(out)), "sf_project")
    return out


def sf_back(g, ig, sino: np.ndarray, bits: int = 64) -> np.ndarray:
    """Adjoint of sf_project: sino (numpy (na, nb)) -> image (numpy (ny, nx))."""
    dt = np.float64 if bits == 64 else np.float32
    sn = np.ascontiguousarray(sino, dtype=dt)
    b, args = _sf_args(g, ig)
    nx, ny = tuple(_f(ig, "dims"))[:2]
    out = np.zeros((int(ny), int(nx)), dtype=dt)
    m = _mask(ig)
    _check(lib(bits).orc_sf_back(*args, _ptr(m), _ptr(sn), _ptr(out)), "sf_back")
    return out


def footprint_size(g, ig) -> float:
    """footprint_size(st, ig), src/sys2/footprint.jl:7-36, as Float32.  fovs(ig) =
    dims .* |deltas| (ImageGeoms 0.11)."""
    d = ig["deltas"]
    di = math.hypot(d[0], d[1])
    rfov = max(ig["dims"][0] * abs(d[0]), ig["dims"][1] * abs(d[1])) / 2
    ct = is_ct(g)
    ratio = di / float(_f(g, "ds") if ct else _f(g, "d"))
    kind = _f(g, "kind")
    if kind == "par":
        return float(np.float32(ratio))
    if rfov > 0.99 * dso(g):
        raise ValueError("bad dso")
    dsd = float(_f(g, "dsd"))
    if kind == "arc":
        return float(np.float32(ratio * dsd / (dso(g) - rfov)))
    smax = float(np.max(np.abs(s_axis(g))))
    return float(np.float32(ratio * math.sqrt(dsd ** 2 + smax ** 2) / (dso(g) - rfov)))
