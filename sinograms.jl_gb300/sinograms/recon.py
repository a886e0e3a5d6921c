"""Reconstruction: plan_fbp / fbp / fdk / cbct_back / fbp_back on the GPU library.

Mirrors src/fbp2/plan2.jl, fbp.jl, fbp-par.jl, back-par.jl, back-fan.jl and
src/fbp3/plan3.jl, fdk.jl, cbct-back.jl.  All arithmetic happens in libsinogb300.so.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._arrays import Arr, check_out, empty, f64, flags_for, is_cuda, out_buffer, plan_call, ptr, stream_for, torch
from .filters import SinogramsArgumentError, Window, fbp_view_weight, fdk_view_weight
from .geom import CtFan, ImageGeom, SinoPar, _ar, _dso, _rfov, c_struct, dims, is_ct


_STORAGE = {"f32": _lib.SGB_STORE_F32, "bf16": _lib.SGB_STORE_BF16, "f16": _lib.SGB_STORE_F16}


def _status(st: int, what: str):
    if st in (_lib.SGB_ERR_ARG, _lib.SGB_ERR_GEOM):
        raise SinogramsArgumentError(f"{what}: {_lib.last_error()}")
    _lib.check(st, what)


class _Plan:
    """Owner of a library plan handle (sgb_plan)."""

    def __init__(self, rg, ig: ImageGeom, window: Window, npad, decon1, filter, storage, source_z=False):
        self.rg, self.ig = rg, ig
        self.window = window
        self.storage = storage
        opts = _lib.FilterOptsC()
        self._keep = []
        if isinstance(window.shape, str):
            opts.window_shape = _lib.SGB_WIN[window.shape]
        else:
            v = f64(window.shape)
            self._keep.append(v)
            opts.window_shape = _lib.SGB_WIN["vect"]
            opts.window_vect = v.ctypes.data
        opts.cutoff = float(window.cutoff)
        opts.npad = int(npad or 0)
        opts.decon1 = int(decon1)
        if filter is not None:
            f = f64(filter)
            self._keep.append(f)
            opts.filter = f.ctypes.data
            opts.npad = len(f)
        opts.storage = _STORAGE[storage]
        opts.source_z = int(bool(source_z))
        self._h = ctypes.c_void_p()
        g, cig = c_struct(rg), ig.c_struct()
        fn = "sgb_plan_fbp_ct" if is_ct(rg) else "sgb_plan_fbp_sino"
        _status(getattr(_lib.lib(), fn)(ctypes.byref(g), ctypes.byref(cig), ctypes.byref(opts),
                                        ctypes.byref(self._h)), "plan_fbp")
        n = ctypes.c_int()
        _status(_lib.lib().sgb_plan_filter(self._h, None, ctypes.byref(n)), "plan_filter")
        self.filter = np.zeros(n.value)
        _status(_lib.lib().sgb_plan_filter(self._h, ptr(self.filter), ctypes.byref(n)), "plan_filter")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib._lib is not None:
            _lib.lib().sgb_plan_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def set_timing(self, enable: bool = True):
        """Record CUDA events around the filter and back-projection stages."""
        _status(_lib.lib().sgb_plan_set_timing(self._h, int(enable)), "plan_set_timing")

    def info(self) -> dict:
        """Execution layout: TMA-staged FDK kernel in use, staged box, row pitch, z-unroll."""
        a = np.zeros(8, dtype=np.int32)
        _status(_lib.lib().sgb_plan_info(self._h, ptr(a), 8), "plan_info")
        return dict(tma=bool(a[0]), box=(int(a[1]), int(a[2])), pitch=int(a[3]), zu=int(a[4]), view_passes=int(a[5]),
                    sample_bytes=int(a[6]), f16_quads=bool(a[7]))

    def set_view_passes(self, passes: int):
        """FDK plans: split the views over `passes` launches (overrides the autotuner's choice)."""
        _status(_lib.lib().sgb_plan_set_view_passes(self._h, int(passes)), "plan_set_view_passes")

    def sync(self):
        """Wait for torch's current stream and raise the device errors of asynchronous calls."""
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _status(_lib.lib().sgb_plan_sync(self._h, st), "plan_sync")

    def last_timing(self):
        """(filter_ms, back_ms) of the last fdk/fbp call (needs set_timing)."""
        ms = np.zeros(2)
        _status(_lib.lib().sgb_plan_last_timing(self._h, ptr(ms), 2), "plan_last_timing")
        return float(ms[0]), float(ms[1])


class FBPNormalPlan(_Plan):
    """FBPNormalPlan (plan2.jl:41-52): rg, ig, filter (Hk), view_weight."""

    @property
    def view_weight(self):
        return fbp_view_weight(self.rg)


class FDKplan(_Plan):
    """FDKplan (plan3.jl:13-23): rg, ig, filter (Hk), view_weight."""

    @property
    def view_weight(self):
        return fdk_view_weight(self.rg)


def plan_fbp(rg, ig: ImageGeom, window: Window = Window(), npad: int | None = None, decon1: bool = True,
             filter=None, storage: str = "f32", source_z: bool = False):
    """plan_fbp(rg, ig; window, npad, decon1, filter), plan2.jl:106-138 / plan3.jl:60-72.

    Additions of this implementation: ``storage`` ("f32", "bf16" or "f16") selects how FDK
    keeps the filtered projections on the GPU (2D plans always use "f32"): "f16" stores each
    detector sample as FP16 terms of its bilinear tap, scaled by a power of two per call; ``source_z=True``
    back-projects a CtSourceHelix scan with t' = mag * (z - source_zs[view]) -- the shift
    the reference leaves commented at cbct-back.jl:188 -- instead of ignoring the source z
    as the reference's cbct_back does."""
    if getattr(rg, "kind", None) == "moj":  # the reference's Mojette plan is commented out (plan2.jl:165-184)
        raise NotImplementedError("plan_fbp: the reference has no FBP for the Mojette geometry (SinoMoj)")
    if is_ct(rg):
        return FDKplan(rg, ig, window, npad, decon1, filter, storage, source_z)
    if source_z:
        raise SinogramsArgumentError("source_z applies to CT (FDK) plans")
    if storage != "f32":
        raise SinogramsArgumentError("2D plans keep filtered sinograms in f32")
    return FBPNormalPlan(rg, ig, window, npad, decon1, filter, storage)


def fdk(plan: FDKplan, proj, out=None, sync: bool = True):
    """image = fdk(plan, proj), fdk.jl:65-81.  proj in numpy order (na, nt, ns) ->
    image (nz, ny, nx).  CUDA tensors stay on the device.  With sync=False the call only
    enqueues its work on torch's current stream, host copies included (plan.sync() waits)."""
    rg = plan.rg
    a = Arr(proj)
    if tuple(reversed(a.shape)) != dims(rg):
        raise SinogramsArgumentError(f"size mismatch {tuple(reversed(a.shape))} {dims(rg)}")  # fdk.jl:68-69
    img = out_buffer(out, tuple(reversed(plan.ig.dims)), a)
    flags, st = plan_call(a.device, sync)
    _status(_lib.lib().sgb_fdk(plan.handle, a.ptr, ptr(img), flags, st), "fdk")
    return img


def _fbp_plan(plan: FBPNormalPlan, sino, out=None, sync=True):
    rg = plan.rg
    a = Arr(sino)
    shp = tuple(reversed(a.shape))  # Julia order (nb, na, ...)
    if shp[:2] != dims(rg):
        raise SinogramsArgumentError("bad sino size")  # fbp.jl:80
    nsl = int(np.prod(shp[2:])) if len(shp) > 2 else 1
    oshape = tuple(reversed(plan.ig.dims)) if len(shp) == 2 else tuple(a.shape[:-2]) + tuple(reversed(plan.ig.dims))
    img = out_buffer(out, oshape, a)
    flags, st = plan_call(a.device, sync)
    _status(_lib.lib().sgb_fbp(plan.handle, a.ptr, ptr(img), nsl, flags, st), "fbp")
    return img


def fbp(plan_or_sino, sino=None, *, out=None, sync=True, **kw):
    """fbp(plan, sino) (fbp.jl:24-68; stacks too) or the convenience fbp(sino; dr, ...)
    (fbp-par.jl:23-36, 63-89)."""
    if isinstance(plan_or_sino, _Plan):
        return _fbp_plan(plan_or_sino, sino, out, sync)
    return _fbp_simple(plan_or_sino, **kw)


def _fbp_simple(sino, nx=None, ny=None, dr=1.0, dx=None, dy=None, orbit=180.0, orbit_start=0.0,
                offset_x=0.0, offset_y=0.0, rmax=0.0, **plan_kw):
    """fbp(sino; dr, ...) -> fbp!, fbp-par.jl:23-89: SinoPar + ImageGeom with a disk mask."""
    a = Arr(sino)
    na, nb = a.shape
    nx = nx or nb
    ny = ny or nx
    dx = dr if dx is None else dx
    dy = dx if dy is None else dy
    rg = SinoPar(nb=nb, na=na, d=dr, orbit=orbit, orbit_start=orbit_start)
    ig = ImageGeom((nx, ny), (dx, dy), (offset_x, offset_y))
    ig = ig.with_mask(ig.circle(_rfov(rg) if rmax == 0 else rmax))
    return _fbp_plan(plan_fbp(rg, ig, **plan_kw), sino)


def cbct_back(proj, rg, ig: ImageGeom, ia_skip: int = 1, sync: bool = True):
    """cbct_back(proj, rg, ig; ia_skip), cbct-back.jl:25-45 (pure back-projection)."""
    if not isinstance(rg, CtFan):
        raise SinogramsArgumentError("cbct_back needs a CtFan geometry")
    if len(ig.dims) != 3:
        raise SinogramsArgumentError("cbct_back needs a 3D ImageGeom")
    a = Arr(proj)
    if tuple(reversed(a.shape)) != dims(rg):  # the view angles come from rg, one per projection
        raise SinogramsArgumentError(f"proj size {tuple(reversed(a.shape))} != dims(rg) {dims(rg)}")
    na, nt, ns = a.shape
    xc, yc, zc = (f64(v) for v in ig.axes())
    betas = f64(_ar(rg))
    mask = None
    if ig.mask is not None:
        mask = Arr(ig.mask if not a.device else __import__("torch").as_tensor(ig.mask, device=a.obj.device),
                   dtype=np.uint8)
    img = empty(tuple(reversed(ig.dims)), a)
    _status(_lib.lib().sgb_cbct_back(ptr(img), a.ptr, ns, nt, na, ptr(betas), rg.dsd, _dso(rg), rg.ds, rg.dt,
                                     rg.offset_s, rg.offset_t, int(rg.kind == "arc"), ptr(xc), ptr(yc), ptr(zc),
                                     ig.dims[0], ig.dims[1], ig.dims[2], None if mask is None else mask.ptr,
                                     ia_skip, flags_for(a.device, sync), stream_for(a.device)), "cbct_back")
    return img


def fbp_back(rg, ig: ImageGeom, sino, ia_skip: int = 1):
    """fbp_back(rg, ig, sino; ia_skip), back-par.jl:184-203 / back-fan.jl:11-32."""
    a = Arr(sino)
    if tuple(reversed(a.shape)) != dims(rg):
        raise SinogramsArgumentError("sino size")
    na, nb = a.shape
    xc, yc = (f64(v) for v in ig.axes())
    ar = _ar(rg)[::ia_skip]
    sn, cs = f64(np.sin(ar)), f64(np.cos(ar))
    mask = None
    if ig.mask is not None:
        mask = Arr(ig.mask if not a.device else __import__("torch").as_tensor(ig.mask, device=a.obj.device),
                   dtype=np.uint8)
    img = empty(tuple(reversed(ig.dims)), a)
    mptr = None if mask is None else mask.ptr
    if rg.kind == "par":
        st = _lib.lib().sgb_fbp_back_par(ptr(img), a.ptr, nb, na, ptr(sn), ptr(cs), rg.d, rg.offset, ptr(xc),
                                         ptr(yc), ig.dims[0], ig.dims[1], mptr, ia_skip, flags_for(a.device),
                                         stream_for(a.device))
    else:
        st = _lib.lib().sgb_fbp_back_fan(ptr(img), a.ptr, nb, na, ptr(sn), ptr(cs), rg.dsd, _dso(rg),
                                         rg.source_offset, int(rg.kind == "arc"), rg.d, rg.offset, ptr(xc),
                                         ptr(yc), ig.dims[0], ig.dims[1], mptr, ia_skip, flags_for(a.device),
                                         stream_for(a.device))
    _status(st, "fbp_back")
    return img


class FDKBatch:
    """Batched FDK: many independent CtFanArc/CtFanFlat scans of different sizes reconstructed
    by one CUDA graph with a single persistent back-projection launch (sgb_batch_fdk_*).
    Each scan's result equals fdk(plan_fbp(rg_i, ig_i), proj_i).  The reference has no
    batched entry point; it reconstructs one scan per `fdk` call (fdk.jl:65-81)."""

    def __init__(self, rgs, igs, window: Window = Window(), npad: int | None = None, decon1: bool = True,
                 storage: str = "f32", source_z: bool = False):
        n = len(rgs)
        if n != len(igs) or n == 0:
            raise SinogramsArgumentError("need one ImageGeom per scan")
        self.rgs, self.igs = list(rgs), list(igs)
        G = (_lib.CtGeomC * n)(*[c_struct(rg) for rg in rgs])
        I = (_lib.ImageGeomC * n)(*[ig.c_struct() for ig in igs])
        opts = _lib.FilterOptsC()
        if not isinstance(window.shape, str):
            raise SinogramsArgumentError("batched FDK takes named windows")
        opts.window_shape = _lib.SGB_WIN[window.shape]
        opts.cutoff = float(window.cutoff)
        opts.npad = int(npad or 0)
        opts.decon1 = int(decon1)
        opts.storage = _STORAGE[storage]
        opts.source_z = int(bool(source_z))
        opts.source_z = int(bool(source_z))
        self._h = ctypes.c_void_p()
        _status(_lib.lib().sgb_batch_fdk_create(n, G, I, ctypes.byref(opts), ctypes.byref(self._h)),
                "batch_fdk_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib._lib is not None:
            _lib.lib().sgb_batch_fdk_destroy(h)
            self._h = None

    def __len__(self):
        return len(self.rgs)

    def set_input(self, i: int, proj):
        a = Arr(proj)
        if tuple(reversed(a.shape)) != dims(self.rgs[i]):
            raise SinogramsArgumentError(f"size mismatch {tuple(reversed(a.shape))} {dims(self.rgs[i])}")
        _status(_lib.lib().sgb_batch_fdk_set_input(self._h, i, a.ptr, flags_for(a.device), stream_for(a.device)),
                "batch_fdk_set_input")

    def get_output(self, i: int, out=None, device: bool = False):
        shape = tuple(reversed(self.igs[i].dims))
        if out is None:
            if device:
                import torch
                out = torch.empty(shape, dtype=torch.float32, device="cuda")
            else:
                out = np.empty(shape, dtype=np.float32)
        dev = is_cuda(out)
        check_out(out, shape, dev)
        _status(_lib.lib().sgb_batch_fdk_get_output(self._h, i, ptr(out), flags_for(dev), stream_for(dev)),
                "batch_fdk_get_output")
        return out

    def run(self, sync: bool = True):
        """fdk of every scan: one CUDA-graph launch on torch's current stream."""
        try:
            import torch
            st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream) if torch.cuda.is_available() else None
        except Exception:
            st = None
        _status(_lib.lib().sgb_batch_fdk_run(self._h, 0 if sync else _lib.SGB_ASYNC, st), "batch_fdk_run")

    def timing(self):
        """Stage times (ms) of the last run: weighted filters, then each persistent launch."""
        n = 1 + self.info()["launches"]
        ms = np.zeros(n)
        _status(_lib.lib().sgb_batch_fdk_timing(self._h, ptr(ms), n), "batch_fdk_timing")
        return [float(v) for v in ms]

    def info(self) -> dict:
        """Totals, and per persistent launch its box class: box width, voxels per thread along
        z, bytes per box sample, views per stage, persistent CTAs, updates (millions) and ring
        stages."""
        u = ctypes.c_longlong()
        a = np.zeros(4 + 7 * 16, dtype=np.int32)
        _status(_lib.lib().sgb_batch_fdk_info(self._h, ctypes.byref(u), ptr(a), len(a)), "batch_fdk_info")
        keys = ("box_width", "zu", "sample_bytes", "views_per_stage", "ctas", "mupdates", "stages")
        classes = [dict(zip(keys, (int(v) for v in a[4 + 7 * c:11 + 7 * c]))) for c in range(int(a[3]))]
        return dict(updates=int(u.value), scans=int(a[0]), work_items=int(a[1]), ctas=int(a[2]), launches=int(a[3]),
                    classes=classes)
