"""Geometries of the golden fixtures and parity cases, as plain parameter dicts.

Shared by tests/golden/make_fixtures.py (oracle side) and the tests (library side), so
both see identical inputs.  ``to_geom`` builds the library's geometry objects.
"""
import math

import numpy as np

ELL3 = np.array([[2.0, 3.0, 1.0, 6.0, 5.0, 4.0, 0.3, 0.4, 0.1, 1.0],
                 [-3.0, -1.0, -2.0, 3.0, 2.0, 4.0, 1.0, 0.2, 0.5, -0.4],
                 [0.0, 0.0, 2.0, 1.5, 1.5, 1.5, 0.0, 0.0, 0.0, 0.8]])
ELL2 = np.array([[1.0, 0.5, 2.0, 1.5, 0.3, 1.0], [-1.0, -1.0, 1.0, 0.7, 1.2, -0.5]])


def gamma_max(g):
    n = g["ns"] if "ns" in g else g["nb"]
    d = g["ds"] if "ns" in g else g["d"]
    off = float(np.float32(g.get("offset_s", g.get("offset", 0.0))))
    s = d * (np.arange(n) - ((n - 1) / 2 + off))
    gam = s / g["dsd"] if g["kind"] == "arc" else np.arctan(s / g["dsd"])
    return float(np.max(np.abs(gam)))


def short(g, na):
    """The `:short` constructor (type2.jl:281-288, type3.jl:333-341)."""
    os_ = 180 + 2 * math.degrees(gamma_max(dict(g, orbit=360.0)))
    return dict(g, na=math.ceil(na * os_ / 360), orbit=os_)


def ct(kind, **kw):
    g = dict(kind=kind, ns=32, nt=24, ds=1.0, dt=1.2, offset_s=0.0, offset_t=0.0, na=24, orbit=360.0,
             orbit_start=0.0, source_offset=0.0, dsd=128.0, dod=32.0)
    g.update(kw)
    return g


FDK_FLAT = dict(rg=ct("flat", offset_s=0.25, offset_t=-0.5),
                ig=dict(dims=(16, 14, 12), deltas=(1.0, 1.1, 0.9), offsets=(0.5, -0.25, 0.3)), window="none")
FDK_ARC_SHORT = dict(rg=short(ct("arc"), 24), ig=dict(dims=(16, 14, 12), deltas=(1.0, 1.0, 1.0)), mask_r=6.0,
                     window="hann", cutoff=0.8)
PAR = dict(rg=dict(kind="par", nb=40, d=0.5, offset=0.25, na=36, orbit=180.0, orbit_start=0.0),
           ig=dict(dims=(24, 20), deltas=(0.5, 0.5)), window="hann")
_ARC = dict(kind="arc", nb=40, d=0.5, offset=0.0, na=48, orbit=360.0, orbit_start=0.0, source_offset=0.0,
            dsd=80.0, dod=20.0)
ARC_SHORT = dict(rg=short(_ARC, 48), ig=PAR["ig"], window="none")
FLAT = dict(rg=dict(_ARC, kind="flat"), ig=PAR["ig"], window="hamming")
BDD = dict(DSD=300.0, DS0=180.0, pSize=2.0, dSize=2.3, nPix=32, nDet=40, angle=np.arange(24) * (2 * math.pi / 24))
FILTER_WRAP = dict(nb=24, npad=32, extra=3, rows=5)
# separable-footprint pair: rectangular pixels, detector and image offsets, a source offset for the fans
SF_IG = dict(dims=(24, 20), deltas=(1.2, 0.9), offsets=(0.5, -0.75))
SF = {kind: dict(rg=dict(kind=kind, nb=40, d=1.1, offset=0.25, na=16, orbit=360.0, orbit_start=10.0,
                         **({} if kind == "par" else dict(dsd=200.0, dod=90.0, source_offset=0.8))), ig=SF_IG)
      for kind in ("par", "arc", "flat")}
# 3D parallel beam (CtPar, type3.jl:102-115): 200 degrees so the Parker ramp of SinoPar applies
CT_PAR = dict(rg=dict(kind="par", ns=40, nt=24, ds=1.0, dt=1.2, offset_s=0.25, offset_t=-0.5, na=40, orbit=200.0,
                      orbit_start=10.0),
              ig=dict(dims=(24, 22, 10), deltas=(1.1, 1.0, 0.9), offsets=(0.3, -0.2, 0.1)))
# helical source (CtSourceHelix, ct-source.jl:29-56): half a zFOV of travel per turn,
# centred so the source z sweeps the image's z extent
HELIX = dict(rg=ct("flat", src="helix", pitch=0.5, source_z0=-5.4, offset_s=0.25),
             ig=dict(dims=(16, 14, 12), deltas=(1.0, 1.1, 0.9), offsets=(0.5, -0.25, 0.3)))


def cyl_mask(ig, r):
    dims, deltas = ig["dims"], ig["deltas"]
    ax = [d * (np.arange(n) - (n - 1) / 2) for n, d in zip(dims, deltas)]
    m2 = (ax[0][None, :] ** 2 + ax[1][:, None] ** 2) <= r * r
    return np.broadcast_to(m2[None], (dims[2],) + m2.shape).copy() if len(dims) == 3 else m2


def to_geom(g):
    """Library geometry object for a parameter dict."""
    import sinograms as S
    g = dict(g)
    kind = g.pop("kind")
    if "ns" in g:
        if g.pop("src", "circle") == "helix":
            g["src"] = S.CtSourceHelix(pitch=g.pop("pitch"), source_z0=g.pop("source_z0"))
        if kind == "par":
            for k in ("dsd", "dod", "source_offset"):
                g.pop(k, None)
            return S.CtPar(**g)
        return (S.CtFanArc if kind == "arc" else S.CtFanFlat)(**g)
    if kind == "par":
        return S.SinoPar(**g)
    return (S.SinoFanArc if kind == "arc" else S.SinoFanFlat)(**g)


def to_image(ig, mask=None):
    import sinograms as S
    return S.ImageGeom(ig["dims"], ig["deltas"], ig.get("offsets"), mask)


def form_bars(storage, na):
    """(relative RMSE, max error / max|ref|) bars of an FDK storage form on an na-view scan.

    FP32 storage: 1e-5 and 1e-4 (FP32 arithmetic against FP64).  A reduced-precision form rounds
    each filtered sample (and, for the F16 quads, the interpolation) independently per view, and a
    voxel sums na views, so its relative error falls as 1/sqrt(na).  The F16 form is held to 1e-4
    at the benchmark's 720 views -- the bound the benchmark's metric states -- scaled by
    sqrt(720 / na); the BF16 form, with three fewer significand bits, to 4e-4 scaled the same way.
    Max error: twice the RMSE bar."""
    if storage == "f32":
        return 1e-5, 1e-4
    k = math.sqrt(720.0 / na) * (1e-4 if storage == "f16" else 4e-4)
    return k, 2 * k
