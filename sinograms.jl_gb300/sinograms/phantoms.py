"""Analytic ellipse / ellipsoid projections on the GPU (the role ImagePhantoms.radon
plays in the reference tests) and the seeded random phantoms of the benchmark configs."""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._arrays import f64, ptr
from .geom import c_struct, is_ct

try:
    import torch
except Exception:  # pragma: no cover
    torch = None


def _project(rg, ell, device):
    ell = f64(ell)
    c = c_struct(rg)
    shape = (rg.na, rg.nt, rg.ns) if is_ct(rg) else (rg.na, rg.nb)
    fn = "sgb_ellipsoid_proj" if is_ct(rg) else "sgb_ellipse_sino"
    nrow = 10 if is_ct(rg) else 6
    nell = ell.size // nrow
    if device:
        out = torch.empty(shape, dtype=torch.float32, device="cuda")
        st = getattr(_lib.lib(), fn)(ctypes.byref(c), ptr(ell), nell, ctypes.c_void_p(out.data_ptr()),
                                     _lib.SGB_DEVICE_PTRS, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    else:
        out = np.empty(shape, dtype=np.float32)
        st = getattr(_lib.lib(), fn)(ctypes.byref(c), ptr(ell), nell, ptr(out), 0, None)
    _lib.check(st, fn)
    return out


def ellipse_sino(rg, ell, device: bool = False):
    """Sinogram (numpy (na, nb)) of ellipses, rows (cx, cy, rx, ry, angle, density)."""
    return _project(rg, ell, device)


def ellipsoid_proj(rg, ell, device: bool = False):
    """Cone-beam projections (numpy (na, nt, ns)) of ellipsoids, rows
    (cx, cy, cz, rx, ry, rz, phi, theta, psi, density) with ZYZ Euler angles."""
    return _project(rg, ell, device)


def random_ellipses(n: int, seed: int, rmax: float, axes=(5.0, 60.0), dens=(-0.5, 1.0)) -> np.ndarray:
    """n ellipses: centres uniform in the disk r <= rmax, semi-axes U[axes], rotation
    U[0, pi), density U[dens]; seeded numpy generator."""
    rng = np.random.default_rng(seed)
    r = rmax * np.sqrt(rng.random(n))
    t = 2 * math.pi * rng.random(n)
    return np.stack([r * np.cos(t), r * np.sin(t), rng.uniform(*axes, n), rng.uniform(*axes, n),
                     rng.uniform(0, math.pi, n), rng.uniform(*dens, n)], axis=1)


def random_ellipsoids(n: int, seed: int, rmax: float, zmax: float, axes=(3.0, 60.0), dens=(-0.3, 1.0)) -> np.ndarray:
    """n ellipsoids: centres uniform in the cylinder r <= rmax, |z| <= zmax, semi-axes
    U[axes], ZYZ Euler angles uniform, density U[dens]."""
    rng = np.random.default_rng(seed)
    r = rmax * np.sqrt(rng.random(n))
    t = 2 * math.pi * rng.random(n)
    return np.stack([r * np.cos(t), r * np.sin(t), rng.uniform(-zmax, zmax, n), rng.uniform(*axes, n),
                     rng.uniform(*axes, n), rng.uniform(*axes, n), rng.uniform(0, 2 * math.pi, n),
                     np.arccos(rng.uniform(-1, 1, n)), rng.uniform(0, 2 * math.pi, n), rng.uniform(*dens, n)], axis=1)


def random_ct_scans(n: int, seed: int, nell: int = 30):
    """n seeded CBCT scans of uneven size (the batched-FDK workload): CtFanFlat or CtFanArc
    50/50, nx = ny in {128..384 step 32}, nz in {128..256 step 32}, na U{180..720},
    ns U{256..768}, nt U{128..384}, dsd U[800,1200], dso = 0.6 dsd, ds = dt = 1; voxels
    sized so the xy square is inscribed in the radial FOV and the slab spans 90% of the
    axial FOV; each scan gets its own random-ellipsoid phantom scaled to its FOV.
    Returns (geometries, image geometries, ellipsoid tables)."""
    from .geom import CtFanArc, CtFanFlat, ImageGeom, _rfov
    rng = np.random.default_rng(seed)
    rgs, igs, ells = [], [], []
    for i in range(n):
        cls = CtFanArc if rng.random() < 0.5 else CtFanFlat
        nx = int(rng.choice(np.arange(128, 385, 32)))
        nz = int(rng.choice(np.arange(128, 257, 32)))
        na, ns, nt = int(rng.integers(180, 721)), int(rng.integers(256, 769)), int(rng.integers(128, 385))
        dsd = float(rng.uniform(800, 1200))
        rg = cls(ns=ns, nt=nt, ds=1.0, dt=1.0, na=na, dsd=dsd, dod=0.4 * dsd)
        rf = _rfov(rg)
        zfov = 0.6 * nt  # dso/dsd * nt * dt (ct-geom.jl:121)
        dx = 2 * rf / (math.sqrt(2) * nx)
        dz = 0.9 * zfov / nz
        rgs.append(rg)
        igs.append(ImageGeom((nx, nx, nz), (dx, dx, dz)))
        e = random_ellipsoids(nell, seed * 1000 + i, 0.6 * rf, 0.35 * nz * dz, axes=(0.02 * rf, 0.3 * rf))
        ells.append(e)
    return rgs, igs, ells
