"""Learned per-row sinogram filter for sparse-view fan-beam FBP (no counterpart in the
reference; it stands in for the apodizing window of fbp_filter, src/fbp/window.jl).

Pipeline (all in libsinogb300.so):
  weighted ramp-filtered rows z = fbp_filter_rows(plan, sino)      (fbp.jl:36, :81-82)
  learned rows               y = z + scale * net(z / scale)       (sgb_lf_apply)
  image                        = fbp_backproject(plan, y)          (back-fan.jl:215-254)
`net` is a 5-layer 1D CNN (kernel 9, 32 channels, GELU; BF16 weights, FP32 master and
accumulation) trained by the library's own forward/backward/Adam kernels to map noisy
ramp-filtered rows onto the ramp-filtered rows of the noise-free data.

The training data are generated here, on the GPU, by the method itself: random-ellipse
phantoms rasterised onto the image grid and projected by the distance-driven projector
(project_bdd, src/sys2/bdd_2d.jl), with Gaussian noise.  The workload's geometry is SinoFanArc;
the reference's projector is flat-detector only (bdd_2d.jl:28-29), so data generation and the
judge use this library's arc-detector form of the pair (BddGeo.arc).

`fbp_learned(..., judge=True)` keeps the learned image only when its reprojection
residual through the same projector does not exceed the plain ramp FBP's by more than
`tol`; otherwise it falls back to plain FBP.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from . import _lib
from ._arrays import Arr, f64, flags_for, ptr, stream_for
from .bdd import BddGeo, BddPlan
from .filters import SinogramsArgumentError
from .geom import ImageGeom, SinoFanArc, SinoFanFlat, _rfov
from .phantoms import random_ellipses
from .recon import FBPNormalPlan, _status, fbp, plan_fbp

try:
    import torch
except Exception:  # pragma: no cover
    torch = None

WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "weights")


def sparse_fan_geometry(na: int = 90, detector: str = "arc"):
    """The sparse-view fan-beam geometry of the learned-filter workload: nb = 888, d = 1.0239,
    dsd = 949.075, dod = 408.075 (the GE LightSpeed values of type2.jl:381-402), na views over
    360 degrees, an arc detector (SinoFanArc; detector="flat" gives SinoFanFlat); 512 x 512 image
    at 0.9766 mm with the FOV disk as mask.  The distance-driven projector that generates the
    training data and judges the result uses the same detector."""
    cls = {"arc": SinoFanArc, "flat": SinoFanFlat}[detector]
    rg = cls(nb=888, d=1.0239, na=na, orbit=360.0, dsd=949.075, dod=408.075)
    ig = ImageGeom((512, 512), (0.9766, 0.9766))
    return rg, ig.with_mask(ig.circle(_rfov(rg)))


# the network's shape: 1 -> 32 -> 32 -> 32 -> 32 -> 1 channels, kernel 9 (W then b per layer)
_CHANNELS = (1, 32, 32, 32, 32, 1)
NPARAM = sum(ci * co * 9 + co for ci, co in zip(_CHANNELS[:-1], _CHANNELS[1:]))


class LearnedFilter:
    """Handle of a learned row filter (sgb_lf)."""

    def __init__(self, scale: float = 1.0, params=None, seed: int = 0):
        self._h = ctypes.c_void_p()
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32).ravel()
        if p is not None and p.size != NPARAM:
            raise ValueError(f"learned filter: {p.size} params given, the network has {NPARAM}")
        _status(_lib.lib().sgb_lf_create(ctypes.c_float(scale), ptr(p), ctypes.c_ulonglong(seed),
                                         ctypes.byref(self._h)), "lf_create")
        self.scale = float(scale)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib._lib is not None:
            _lib.lib().sgb_lf_destroy(h)
            self._h = None

    @property
    def nparam(self) -> int:
        return int(_lib.lib().sgb_lf_num_params(self._h))

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparam, dtype=np.float32)
        _status(_lib.lib().sgb_lf_get_params(self._h, ptr(out), None), "lf_get_params")
        return out

    def save(self, path: str):
        np.savez(path, params=self.params(), scale=np.float32(self.scale))

    @classmethod
    def load(cls, path: str):
        d = np.load(path)
        return cls(float(d["scale"]), d["params"])

    def adam_state(self):
        """(m, v, step): the Adam moments (FP32, the params' layout) and the steps taken."""
        m = np.zeros(self.nparam, dtype=np.float32)
        v = np.zeros(self.nparam, dtype=np.float32)
        step = ctypes.c_longlong()
        _status(_lib.lib().sgb_lf_get_state(self._h, ptr(m), ptr(v), ctypes.byref(step)), "lf_get_state")
        return m, v, int(step.value)

    def set_adam_state(self, m, v, step: int):
        m = np.ascontiguousarray(m, dtype=np.float32)
        v = np.ascontiguousarray(v, dtype=np.float32)
        if m.size != self.nparam or v.size != self.nparam:
            raise ValueError(f"Adam state of {m.size}/{v.size} values for a filter of {self.nparam} params")
        _status(_lib.lib().sgb_lf_set_state(self._h, ptr(m), ptr(v), int(step)), "lf_set_state")

    def save_checkpoint(self, path: str):
        """Params, scale and Adam state: load_checkpoint(path) resumes training where it stopped."""
        m, v, step = self.adam_state()
        np.savez(path, params=self.params(), scale=np.float32(self.scale), adam_m=m, adam_v=v,
                 adam_step=np.int64(step))

    @classmethod
    def load_checkpoint(cls, path: str):
        d = np.load(path)
        lf = cls(float(d["scale"]), d["params"])
        lf.set_adam_state(d["adam_m"], d["adam_v"], int(d["adam_step"]))
        return lf

    def apply(self, z, sync: bool = True):
        """y = z + scale * net(z / scale) for rows z of shape (..., L); with CUDA tensors and
        sync=False the call only enqueues work on the current stream."""
        a = Arr(z)
        L = a.shape[-1]
        R = int(np.prod(a.shape[:-1]))
        out = torch.empty(a.shape, dtype=torch.float32, device=a.obj.device) if a.device else np.empty(a.shape,
                                                                                                        np.float32)
        for r0 in range(0, R, 65535):
            n = min(65535, R - r0)
            zi = ctypes.c_void_p(a.ptr.value + 4 * r0 * L)
            yi = ctypes.c_void_p(ptr(out).value + 4 * r0 * L)
            _status(_lib.lib().sgb_lf_apply(self._h, zi, n, L, yi, flags_for(a.device, sync), stream_for(a.device)),
                    "lf_apply")
        return out

    def loss_grad(self, z, target, grads: bool = True):
        a, t = Arr(z), Arr(target)
        L = a.shape[-1]
        R = int(np.prod(a.shape[:-1]))
        loss = ctypes.c_double()
        g = np.zeros(self.nparam, dtype=np.float32) if grads else None
        _status(_lib.lib().sgb_lf_loss_grad(self._h, a.ptr, t.ptr, R, L, ctypes.byref(loss), ptr(g),
                                            flags_for(a.device), stream_for(a.device)), "lf_loss_grad")
        return (loss.value, g) if grads else loss.value

    def train_step(self, z, target, lr: float) -> float:
        a, t = Arr(z), Arr(target)
        L = a.shape[-1]
        R = int(np.prod(a.shape[:-1]))
        loss = ctypes.c_double()
        _status(_lib.lib().sgb_lf_train_step(self._h, a.ptr, t.ptr, R, L, ctypes.c_float(lr), ctypes.byref(loss),
                                             flags_for(a.device), stream_for(a.device)), "lf_train_step")
        return loss.value


# ------------------------------------------------------------------- plan stages

def fbp_filter_rows(plan: FBPNormalPlan, sino, sync: bool = True):
    """Weighted, ramp-filtered rows of fbp(plan, sino) (the stage before back-projection)."""
    a = Arr(sino)
    out = torch.empty(a.shape, dtype=torch.float32, device=a.obj.device) if a.device else np.empty(a.shape, np.float32)
    nsl = int(np.prod(a.shape[:-2])) if len(a.shape) > 2 else 1
    _status(_lib.lib().sgb_fbp_filter_rows(plan.handle, a.ptr, ptr(out), nsl, flags_for(a.device, sync),
                                           stream_for(a.device)), "fbp_filter_rows")
    return out


def fbp_backproject(plan: FBPNormalPlan, filtered, sync: bool = True):
    """The back-projection stage of fbp(plan, sino) on already filtered rows."""
    a = Arr(filtered)
    shape = tuple(a.shape[:-2]) + tuple(reversed(plan.ig.dims))
    out = torch.empty(shape, dtype=torch.float32, device=a.obj.device) if a.device else np.empty(shape, np.float32)
    nsl = int(np.prod(a.shape[:-2])) if len(a.shape) > 2 else 1
    _status(_lib.lib().sgb_fbp_backproject(plan.handle, a.ptr, ptr(out), nsl, flags_for(a.device, sync),
                                           stream_for(a.device)), "fbp_backproject")
    return out


# ---------------------------------------------------------- phantoms and data

def ellipse_image(ig: ImageGeom, ell, sub: int = 2, device: bool = True):
    """Pixel image of ellipses on ig (numpy order (ny, nx)), sub x sub samples per pixel."""
    e = f64(ell)
    c = ig.c_struct()
    shape = tuple(reversed(ig.dims))
    if device:
        out = torch.empty(shape, dtype=torch.float32, device="cuda")
        st = _lib.lib().sgb_ellipse_image(ctypes.byref(c), ptr(e), e.size // 6, sub, ctypes.c_void_p(out.data_ptr()),
                                          _lib.SGB_DEVICE_PTRS,
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    else:
        out = np.empty(shape, dtype=np.float32)
        st = _lib.lib().sgb_ellipse_image(ctypes.byref(c), ptr(e), e.size // 6, sub, ptr(out), 0, None)
    _lib.check(st, "ellipse_image")
    return out


def image_to_dd(img):
    """ImageGeom-order image (ny, nx) -> project_bdd phantom layout (Julia (nPix,nPix), row 1
    = top = largest y), as test/sys2/bdd_2d.jl:31 does with reverse(rot180(img'), dims=2)."""
    return torch.flip(img, dims=[0]).T.contiguous()


_BDD_PLANS: dict = {}


def bdd_plan(geo: BddGeo) -> BddPlan:
    """The cached projector plan of a geo tuple (the data generator and the judge project
    many images through one geometry)."""
    ang = f64(geo.angle)
    key = (float(geo.DSD), float(geo.DS0), float(geo.pSize), float(geo.dSize), int(geo.nPix), int(geo.nDet),
           ang.tobytes(), bool(getattr(geo, "arc", False)))
    plan = _BDD_PLANS.get(key)
    if plan is None:
        if len(_BDD_PLANS) >= 8:
            _BDD_PLANS.clear()
        plan = _BDD_PLANS[key] = BddPlan(geo)
    return plan


def dd_project(img, geo: BddGeo, sync: bool = True):
    """DD sinogram of an ImageGeom-order image, returned in FBP order (na, nb)."""
    return bdd_plan(geo).project(image_to_dd(img), sync=sync).T.contiguous()


def phantom_ellipses(seed: int, n: int = 20):
    """The seeded random-ellipse phantoms of the fan-beam workloads: centres in the disk
    r <= 220 mm, semi-axes U[4, 120] mm, rotation U[0, pi), density U[-0.3, 1.0]."""
    return random_ellipses(n, seed, 220.0, axes=(4.0, 120.0), dens=(-0.3, 1.0))


def make_dataset(n_phantoms: int, seed: int, rg=None, ig=None, noise: float = 0.005, chunk: int = 64):
    """Training rows on the GPU: (z_noisy, z_clean, images, sinos) where z are the plan's
    weighted ramp-filtered rows (n_phantoms*na, nb) of the DD sinograms with and without
    Gaussian noise of sigma = noise * max(sinogram)."""
    if rg is None:
        rg, ig = sparse_fan_geometry()
    plan = plan_fbp(rg, ig)
    geo = BddGeo.from_geoms(rg, ig)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    zn = torch.empty((n_phantoms, rg.na, rg.nb), device="cuda")
    zc = torch.empty_like(zn)
    ig0 = ig.with_mask(None)
    for p0 in range(0, n_phantoms, chunk):
        p1 = min(n_phantoms, p0 + chunk)
        s = torch.empty((p1 - p0, rg.na, rg.nb), device="cuda")
        for i in range(p0, p1):
            s[i - p0] = dd_project(ellipse_image(ig0, phantom_ellipses(seed * 100003 + i)), geo)
        peak = s.abs().amax(dim=(1, 2), keepdim=True)
        sn = s + noise * peak * torch.randn(s.shape, device="cuda", generator=gen)
        zc[p0:p1] = fbp_filter_rows(plan, s)
        zn[p0:p1] = fbp_filter_rows(plan, sn)
    return zn.reshape(-1, rg.nb), zc.reshape(-1, rg.nb)


def train(lf: LearnedFilter, zn, zc, epochs: int = 2, batch: int = 4096, lr: float = 1e-3, seed: int = 0,
          log=None, start: int = 0, stop: int | None = None):
    """Adam over shuffled row batches with a cosine-decayed rate; returns the per-step losses.
    Runs steps start .. stop-1 of the epochs * (rows // batch) step schedule, so a filter saved by
    save_checkpoint after k steps and restored by load_checkpoint continues with start = k (the
    shuffles of the epochs already done are drawn again from the seeded generator, on the
    rows' device)."""
    dev = zn.device
    g = torch.Generator(device=dev).manual_seed(seed)
    R = zn.shape[0]
    per = R // batch
    losses = []
    steps = epochs * per
    stop = steps if stop is None else min(stop, steps)
    for _ in range(start // per):
        torch.randperm(R, device=dev, generator=g)
    perm = None
    for step in range(start, stop):
        j = step % per
        if j == 0 or perm is None:
            perm = torch.randperm(R, device=dev, generator=g)
        idx = perm[j * batch:(j + 1) * batch]
        rate = lr * 0.5 * (1 + math.cos(math.pi * step / steps))  # cosine decay
        losses.append(lf.train_step(zn[idx].contiguous(), zc[idx].contiguous(), max(rate, 1e-6)))
        if log and step % 50 == 0:
            log(step, losses[-1])
    return losses


# ------------------------------------------------------------------ inference

def reprojection_residual(img, sino, geo: BddGeo) -> float:
    """||A x - y|| / ||y|| with A the distance-driven projector."""
    r = dd_project(img, geo) - sino
    return float(r.norm() / sino.norm())


def fbp_learned(plan: FBPNormalPlan, lf: LearnedFilter, sino, judge: bool = True, tol: float = 0.0):
    """FBP with the learned row filter.  With judge=True both the learned and the plain
    ramp images are reprojected by the DD projector; the learned image is returned only if
    its residual is at most (1 + tol) times the plain one, else plain FBP (fallback).
    Returns (image, info)."""
    z = fbp_filter_rows(plan, sino)
    img_l = fbp_backproject(plan, lf.apply(z))
    if not judge:
        return img_l, {"used": "learned"}
    img_p = fbp_backproject(plan, z)
    geo = BddGeo.from_geoms(plan.rg, plan.ig)
    rl = reprojection_residual(img_l, sino, geo)
    rp = reprojection_residual(img_p, sino, geo)
    used = "learned" if rl <= (1 + tol) * rp else "plain"
    return (img_l if used == "learned" else img_p), {"used": used, "residual_learned": rl, "residual_plain": rp}


# ------------------------------------------------------ learned linear (ramp) filter

class LearnedRamp:
    """Learned linear row filter: the plan's ramp response Hk times a per-frequency gain G(k)
    fitted on the same self-generated data as the CNN.  G is the least-squares optimum over all
    real, even, shift-invariant row filters for the CNN's loss (filtered noisy rows against the
    filtered noise-free rows, evaluated over the full padded row):

        G(k) = sum Re(conj(Wn(k)) Wc(k)) / sum |Wn(k)|^2,

    with Wn, Wc the length-npad FFTs of the zero-padded weighted noisy and noise-free rows (the
    ramp factor cancels).  Because G only changes the plan's Hk (the `filter` option of plan_fbp,
    plan2.jl:106-138), FBP with it runs exactly the plain FBP kernels: same launches, same
    latency."""

    def __init__(self, gain, npad: int, meta: dict | None = None):
        self.gain = np.asarray(gain, dtype=np.float64)
        if self.gain.shape != (npad,):
            raise SinogramsArgumentError(f"gain has shape {self.gain.shape}, expected ({npad},)")
        self.npad = int(npad)
        self.meta = dict(meta or {})

    def plan(self, rg, ig, window=None):
        """plan_fbp(rg, ig; filter = Hk .* G) with Hk the plan's own ramp response."""
        base = plan_fbp(rg, ig, npad=self.npad) if window is None else plan_fbp(rg, ig, window=window,
                                                                                npad=self.npad)
        return plan_fbp(rg, ig, filter=base.filter * self.gain)

    def save(self, path: str):
        np.savez(path, gain=self.gain, npad=np.int64(self.npad),
                 **{k: np.asarray(v) for k, v in self.meta.items()})

    @classmethod
    def load(cls, path: str):
        d = np.load(path)
        meta = {k: d[k].item() for k in d.files if k not in ("gain", "npad")}
        return cls(d["gain"], int(d["npad"]), meta)


def fit_learned_ramp(n_phantoms: int, seed: int, rg=None, ig=None, noise: float = 0.005,
                     chunk: int = 64) -> LearnedRamp:
    """Fit G(k) on n_phantoms seeded random-ellipse scans (the CNN's data: DD projections
    plus Gaussian noise of sigma = noise * max(sinogram)).  The weighted rows come from an
    all-pass plan (Hk = 1), whose filtered rows are the weighted sinogram itself; the spectra
    are accumulated in float64 on the host."""
    if rg is None:
        rg, ig = sparse_fan_geometry()
    base = plan_fbp(rg, ig)
    npad = len(base.filter)
    allpass = plan_fbp(rg, ig, filter=np.ones(npad))
    geo = BddGeo.from_geoms(rg, ig)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    ig0 = ig.with_mask(None)
    cross = np.zeros(npad // 2 + 1)
    power = np.zeros(npad // 2 + 1)
    for p0 in range(0, n_phantoms, chunk):
        p1 = min(n_phantoms, p0 + chunk)
        s = torch.empty((p1 - p0, rg.na, rg.nb), device="cuda")
        for i in range(p0, p1):
            s[i - p0] = dd_project(ellipse_image(ig0, phantom_ellipses(seed * 100003 + i)), geo)
        peak = s.abs().amax(dim=(1, 2), keepdim=True)
        sn = s + noise * peak * torch.randn(s.shape, device="cuda", generator=gen)
        wc = fbp_filter_rows(allpass, s).reshape(-1, rg.nb).cpu().numpy().astype(np.float64)
        wn = fbp_filter_rows(allpass, sn).reshape(-1, rg.nb).cpu().numpy().astype(np.float64)
        fc = np.fft.rfft(wc, n=npad, axis=1)
        fn = np.fft.rfft(wn, n=npad, axis=1)
        cross += np.sum((fn.conj() * fc).real, axis=0)
        power += np.sum(np.abs(fn) ** 2, axis=0)
    half = np.where(power > 0, cross / np.where(power > 0, power, 1.0), 1.0)
    gain = np.concatenate([half, half[1:npad - npad // 2][::-1]])  # even: G(npad - k) = G(k)
    return LearnedRamp(gain, npad, {"phantoms": n_phantoms, "seed": seed, "noise": noise})


def fbp_learned_ramp(plan_learned: FBPNormalPlan, plan_plain: FBPNormalPlan, sino, judge: bool = True,
                     tol: float = 0.0):
    """FBP through the learned-ramp plan, judged as fbp_learned judges the CNN: the learned
    image is kept only if its DD reprojection residual is at most (1 + tol) times plain ramp
    FBP's, else plain FBP is returned.  Returns (image, info)."""
    img_l = fbp(plan_learned, sino)
    if not judge:
        return img_l, {"used": "learned"}
    img_p = fbp(plan_plain, sino)
    geo = BddGeo.from_geoms(plan_plain.rg, plan_plain.ig)
    rl = reprojection_residual(img_l, sino, geo)
    rp = reprojection_residual(img_p, sino, geo)
    used = "learned" if rl <= (1 + tol) * rp else "plain"
    return (img_l if used == "learned" else img_p), {"used": used, "residual_learned": rl, "residual_plain": rp}


def default_ramp_path(detector: str = "arc") -> str:
    return os.path.join(WEIGHTS_DIR, f"learned_ramp_fan{detector}888_90v.npz")


def default_weights_path(detector: str = "arc") -> str:
    return os.path.join(WEIGHTS_DIR, f"learned_filter_fan{detector}888_90v.npz")
