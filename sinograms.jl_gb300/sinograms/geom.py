"""Ray and image geometries, mirroring Sinograms.jl's geometry types.

Fields and keyword defaults follow src/geom/type2.jl (SinoPar, SinoFanArc, SinoFanFlat)
and src/geom/type3.jl (CtFanArc, CtFanFlat); helper functions follow
src/geom/common.jl, sino-geom.jl and ct-geom.jl.  Lengths are plain floats (no Unitful);
angles are in degrees like the reference's defaults.  Offsets are rounded to Float32
as the reference stores them (Toffset = Float32, src/geom/util.jl:5).

Array convention of this package: numpy/torch arrays are C-ordered with the Julia
dimensions reversed, so memory matches the reference's column-major arrays exactly:
sinogram (nb, na) is ``(na, nb)``, projections (ns, nt, na) are ``(na, nt, ns)`` and an
image (nx, ny[, nz]) is ``([nz,] ny, nx)``.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import _lib


def _f32(x) -> float:
    return float(np.float32(x))


def _default_na(nb: int) -> int:
    return 2 * math.floor(nb * math.pi / 2 / 2)  # type2.jl:186


@dataclass(frozen=True)
class SinoPar:
    """2D parallel-beam sinogram geometry (type2.jl:95-104, constructor :182-195)."""
    nb: int = 128
    d: float = 1.0
    offset: float = 0.0
    na: int | None = None
    orbit: float = 180.0
    orbit_start: float = 0.0
    kind = "par"

    def __post_init__(self):
        object.__setattr__(self, "offset", _f32(self.offset))
        if self.na is None:
            object.__setattr__(self, "na", _default_na(self.nb))


@dataclass(frozen=True)
class SinoMoj:
    """2D Mojette sinogram geometry (type2.jl:112-121, constructor :215-229).  ``d`` is the
    square pixel size; a view at angle phi samples rays d * max(|cos phi|, |sin phi|) apart
    (_d_moj, common.jl:128).  The reference gives it a ramp (fbp_ramp with ``dr``, ramp.jl:27-30)
    and a Parker weight (parker.jl:122-129) but no reconstruction: its Mojette plan is commented
    out (plan2.jl:165-184), so plan_fbp refuses it here as well."""
    nb: int = 128
    d: float = 1.0
    offset: float = 0.0
    na: int | None = None
    orbit: float = 180.0
    orbit_start: float = 0.0
    kind = "moj"

    def __post_init__(self):
        object.__setattr__(self, "offset", _f32(self.offset))
        if self.na is None:
            object.__setattr__(self, "na", _default_na(self.nb))


@dataclass(frozen=True)
class _SinoFan:
    nb: int = 128
    d: float = 1.0
    offset: float = 0.0
    na: int | None = None
    orbit: float = 360.0
    orbit_start: float = 0.0
    source_offset: float = 0.0
    dsd: float | None = None
    dod: float | None = None

    def __post_init__(self):
        object.__setattr__(self, "offset", _f32(self.offset))
        if self.na is None:
            object.__setattr__(self, "na", _default_na(self.nb))
        if self.dsd is None:
            object.__setattr__(self, "dsd", 4 * self.nb * self.d)  # type2.jl:267
        if self.dod is None:
            object.__setattr__(self, "dod", self.nb * self.d)

    @classmethod
    def short(cls, na: int = 128, orbit_start: float = 0.0, **kw):
        """`SinoFanArc(:short; ...)`, type2.jl:281-288: orbit = 180 + fan angle, na scaled."""
        tmp = cls(orbit=360.0, **kw)
        os_ = _orbit_short(tmp)
        return cls(na=math.ceil(na * os_ / 360), orbit=os_, orbit_start=orbit_start, **kw)


@dataclass(frozen=True)
class SinoFanArc(_SinoFan):
    """2D fan-beam geometry with an arc detector (type2.jl:128-140)."""
    kind = "arc"

    @classmethod
    def ge1(cls, orbit="360", **kw):
        """GE LightSpeed preset, `SinoFanArc(Val(:ge1))`, type2.jl:381-402."""
        args = dict(nb=888, d=1.0239, offset=1.25, na=984, orbit=360.0, dsd=949.075, dod=408.075)
        if orbit == "short":
            args["na"] = 642
            args["orbit"] = _f32(642 / 984 * 360)
        args.update(kw)
        return cls(**args)


@dataclass(frozen=True)
class SinoFanFlat(_SinoFan):
    """2D fan-beam geometry with a flat detector (type2.jl:147-159)."""
    kind = "flat"


@dataclass(frozen=True)
class CtSourceCircle:
    """Circular source trajectory (src/geom/ct-source.jl:22-26)."""


@dataclass(frozen=True)
class CtSourceHelix:
    """Helical source with constant pitch (src/geom/ct-source.jl:29-56): ``pitch`` is a
    Float32 fraction of the z field of view per turn, ``source_z0`` the first view's z."""
    pitch: float = 0.0
    source_z0: float = 0.0

    def __post_init__(self):
        object.__setattr__(self, "pitch", _f32(self.pitch))


@dataclass(frozen=True)
class _CtFan:
    ns: int = 128
    nt: int = 64
    ds: float = 1.0
    dt: float | None = None
    offset_s: float = 0.0
    offset_t: float = 0.0
    na: int = 64
    orbit: float = 360.0
    orbit_start: float = 0.0
    source_offset: float = 0.0
    dsd: float | None = None
    dod: float | None = None
    src: object = CtSourceCircle()

    def __post_init__(self):
        object.__setattr__(self, "offset_s", _f32(self.offset_s))
        object.__setattr__(self, "offset_t", _f32(self.offset_t))
        if self.dt is None:
            object.__setattr__(self, "dt", self.ds)
        if self.dsd is None:
            object.__setattr__(self, "dsd", 4 * self.ns * self.ds)  # type3.jl:317
        if self.dod is None:
            object.__setattr__(self, "dod", self.ns * self.ds)

    @classmethod
    def short(cls, na: int = 128, orbit_start: float = 0.0, **kw):
        """`CtFanArc(:short; ...)`, type3.jl:333-341."""
        tmp = cls(orbit=360.0, **kw)
        os_ = _orbit_short(tmp)
        return cls(na=math.ceil(na * os_ / 360), orbit=os_, orbit_start=orbit_start, **kw)


@dataclass(frozen=True)
class CtFanArc(_CtFan):
    """3D cone-beam geometry with an arc detector (type3.jl:145-161)."""
    kind = "arc"

    @classmethod
    def ge1(cls, orbit="360", **kw):
        """GE LightSpeed preset, `CtFanArc(Val(:ge1))`, type3.jl:443-467."""
        args = dict(ns=888, nt=64, ds=1.0239, dt=1.0964, offset_s=1.25, na=984, orbit=360.0, dsd=949.075,
                    dod=408.075)
        if orbit == "short":
            args["na"] = 642
            args["orbit"] = 642 / 984 * 360
        args.update(kw)
        return cls(**args)


@dataclass(frozen=True)
class CtFanFlat(_CtFan):
    """3D cone-beam geometry with a flat detector (type3.jl:168-184)."""
    kind = "flat"


@dataclass(frozen=True)
class CtPar:
    """3D parallel-beam geometry (type3.jl:102-115, constructor defaults :211-230).  The
    reference defines it but has no FBP for it; plan_fbp(CtPar, ig) + fdk here reconstruct
    it with the flat ramp, SinoPar's view weights and a voxel-driven back-projection with
    s = x cos(b) + y sin(b) and t = z."""
    ns: int = 128
    nt: int = 64
    ds: float = 1.0
    dt: float | None = None
    offset_s: float = 0.0
    offset_t: float = 0.0
    na: int = 60
    orbit: float = 180.0
    orbit_start: float = 0.0
    kind = "par"
    src = CtSourceCircle()
    source_offset = 0.0
    dsd = 0.0
    dod = 0.0

    def __post_init__(self):
        object.__setattr__(self, "offset_s", _f32(self.offset_s))
        object.__setattr__(self, "offset_t", _f32(self.offset_t))
        if self.dt is None:
            object.__setattr__(self, "dt", self.ds)


SinoGeom = (SinoPar, SinoFanArc, SinoFanFlat)
SinoFan = (SinoFanArc, SinoFanFlat)
CtFan = (CtFanArc, CtFanFlat)
CtGeom = (CtFanArc, CtFanFlat, CtPar)


def is_ct(rg) -> bool:
    return isinstance(rg, CtGeom)


def dims(rg):
    """dims(rg), sino-geom.jl:13 / ct-geom.jl:14 (Julia order)."""
    return (rg.ns, rg.nt, rg.na) if is_ct(rg) else (rg.nb, rg.na)


def angles(rg) -> np.ndarray:
    """angles(rg) in degrees, common.jl:27-28."""
    return rg.orbit_start + np.arange(rg.na) * (rg.orbit / rg.na)


def _ar(rg) -> np.ndarray:
    """Angles in radians, common.jl:34."""
    return angles(rg) * (math.pi / 180)


def _s(rg) -> np.ndarray:
    """Detector s sample positions, sino-geom.jl:18-20 / ct-geom.jl:19-23."""
    if is_ct(rg):
        return rg.ds * (np.arange(rg.ns) - ((rg.ns - 1) / 2 + rg.offset_s))
    return rg.d * (np.arange(rg.nb) - ((rg.nb - 1) / 2 + rg.offset))


def _t(rg) -> np.ndarray:
    return rg.dt * (np.arange(rg.nt) - ((rg.nt - 1) / 2 + rg.offset_t))


def _d_ang(rg: SinoMoj) -> np.ndarray:
    """Ray spacing of each Mojette view, d * max(|cos|, |sin|) of its angle (common.jl:128-129)."""
    ar = _ar(rg)
    return rg.d * np.maximum(np.abs(np.cos(ar)), np.abs(np.sin(ar)))


def _ds(rg) -> float:
    return rg.ds if is_ct(rg) else rg.d


def _dso(rg) -> float:
    return rg.dsd - rg.dod


def _gamma(rg) -> np.ndarray:
    s = _s(rg)
    return s / rg.dsd if rg.kind == "arc" else np.arctan(s / rg.dsd)


def _gamma_max(rg) -> float:
    return float(np.max(np.abs(_gamma(rg))))


def _orbit_short(rg) -> float:
    return 180 + 2 * math.degrees(_gamma_max(rg))


def _rfov(rg) -> float:
    """Radial FOV, common.jl:59-61."""
    if rg.kind == "par":
        return float(np.max(np.abs(_s(rg))))
    return _dso(rg) * math.sin(_gamma_max(rg))


def downsample(rg, down: int):
    """downsample(rg, down), sino-geom.jl:32-53 / ct-geom.jl:28-55."""
    if down == 1:
        return rg
    if is_ct(rg):
        return replace(rg, ns=4 * max(rg.ns // (4 * down), 1), nt=2 * max(rg.nt // (2 * down), 1),
                       ds=rg.ds * down, dt=rg.dt * down, na=max(rg.na // down, 1))
    return replace(rg, nb=2 * max(rg.nb // (2 * down), 1), d=rg.d * down, na=max(rg.na // down, 1))


def _zfov(rg) -> float:
    """_zfov(rg), ct-geom.jl:119-121."""
    if isinstance(rg, CtPar):
        return rg.nt * rg.dt
    return _dso(rg) / rg.dsd * rg.nt * rg.dt


def _source_dz_per_view(rg) -> float:
    """_source_dz_per_view(rg), ct-geom.jl:123-131."""
    if not isinstance(rg.src, CtSourceHelix) or rg.na == 1:
        return 0.0
    return rg.src.pitch * _zfov(rg) / (rg.na * (360 / rg.orbit))


def _source_zs(rg) -> np.ndarray:
    """_source_zs(rg), ct-geom.jl:134-140 (computed by the library's host code)."""
    zs = np.zeros(rg.na)
    _lib.check(_lib.lib().sgb_source_zs(ctypes.byref(c_struct(rg)), zs.ctypes.data), "source_zs")
    return zs


def c_struct(rg):
    """The C ABI struct (sgb_sino_geom / sgb_ct_geom) for a geometry."""
    kinds = {"par": _lib.SGB_PAR, "arc": _lib.SGB_ARC, "flat": _lib.SGB_FLAT}
    if rg.kind not in kinds:
        raise ValueError(f"{type(rg).__name__} has no reconstruction in the library")
    kind = kinds[rg.kind]
    if is_ct(rg):
        helix = isinstance(rg.src, CtSourceHelix)
        return _lib.CtGeomC(kind, rg.ns, rg.nt, rg.ds, rg.dt, rg.offset_s, rg.offset_t, rg.na, rg.orbit,
                            rg.orbit_start, rg.source_offset, rg.dsd, rg.dod,
                            _lib.SGB_SRC_HELIX if helix else _lib.SGB_SRC_CIRCLE,
                            rg.src.pitch if helix else 0.0, rg.src.source_z0 if helix else 0.0)
    return _lib.SinoGeomC(kind, rg.nb, rg.d, rg.offset, rg.na, rg.orbit, rg.orbit_start,
                          getattr(rg, "source_offset", 0.0), getattr(rg, "dsd", 0.0) or 0.0,
                          getattr(rg, "dod", 0.0) or 0.0)


@dataclass
class ImageGeom:
    """ImageGeom (ImageGeoms.jl 0.11): dims, deltas, offsets and an optional mask.

    Pixel centres are ``delta * (i - (n+1)/2 - offset)`` for i = 1..n.  ``mask`` is a bool
    array in this package's numpy order (reversed dims) or None for all-true.
    """
    dims: tuple
    deltas: tuple = None
    offsets: tuple = None
    mask: np.ndarray | None = field(default=None, repr=False)

    def __post_init__(self):
        self.dims = tuple(int(n) for n in self.dims)
        nd = len(self.dims)
        self.deltas = tuple(float(d) for d in (self.deltas or (1.0,) * nd))
        self.offsets = tuple(float(o) for o in (self.offsets or (0.0,) * nd))
        if self.mask is not None:
            m = np.asarray(self.mask, dtype=bool)
            if m.shape != tuple(reversed(self.dims)):
                raise ValueError(f"mask shape {m.shape} != {tuple(reversed(self.dims))}")
            self.mask = m

    @property
    def ndim(self) -> int:
        return len(self.dims)

    def axes(self):
        return [d * (np.arange(n) - ((n - 1) / 2 + o)) for n, d, o in zip(self.dims, self.deltas, self.offsets)]

    def circle(self, r: float) -> np.ndarray:
        """Disk/cylinder mask x^2 + y^2 <= r^2 in numpy order (the ImageGeoms `circle`)."""
        ax = self.axes()
        m2 = (ax[0][None, :] ** 2 + ax[1][:, None] ** 2) <= r * r
        if self.ndim == 3:
            m2 = np.broadcast_to(m2[None], (self.dims[2],) + m2.shape).copy()
        return m2

    def with_mask(self, mask) -> "ImageGeom":
        return ImageGeom(self.dims, self.deltas, self.offsets, mask)

    def c_struct(self):
        c = _lib.ImageGeomC()
        c.ndim = self.ndim
        for i in range(self.ndim):
            c.dims[i], c.deltas[i], c.offsets[i] = self.dims[i], self.deltas[i], self.offsets[i]
        self._mask_u8 = None if self.mask is None else np.ascontiguousarray(self.mask, dtype=np.uint8)
        c.mask = None if self._mask_u8 is None else self._mask_u8.ctypes.data
        return c


def axes(ig: ImageGeom):
    return ig.axes()
