"""Parity at the full benchmark sizes.

* CBCT flat panel (CtFanFlat 512x384x720 -> 512x512x256, the benchmark): every 16th voxel in x and
  y on every 32nd slice against the FP64 oracle (the oracle filters every detector row by
  FFT and back-projects the sampled voxels), for the FP32 form and the F16 storage form; exact
  scaling fdk(2p) == 2 fdk(p) and additivity on the whole volume;
* 2D parallel beam (SinoPar 256 x 180, Hann) and 2D fan arc (SinoFanArc 888 x 512 views over a short
  scan, Parker, noisy): whole images against the FP64 oracle, compared inside the
  reconstruction FOV."""
import math
import os

import numpy as np
import pytest

import oracle as O
import sinograms as S

pytestmark = pytest.mark.gpu

GEOM3 = dict(ns=512, nt=384, ds=1.0, dt=1.0, dsd=1000.0, dod=400.0, na=720, orbit=360.0)


def _workers():
    return os.cpu_count() or 1


@pytest.fixture(scope="module")
def cbct_flat_512(cuda):
    import torch
    rg = S.CtFanFlat(**GEOM3)
    ig = S.ImageGeom((512, 512, 256), (0.5, 0.5, 0.5))
    ell = S.random_ellipsoids(30, 3, 100.0, 50.0, axes=(3.0, 60.0), dens=(-0.3, 1.0))
    proj = S.ellipsoid_proj(rg, ell, device=True)
    plan = S.plan_fbp(rg, ig)
    img = S.fdk(plan, proj)
    torch.cuda.synchronize()
    return rg, ig, plan, proj, img


@pytest.fixture(scope="module")
def cbct_flat_512_ref(cbct_flat_512):
    """FP64 oracle on a sparse sample of the benchmark volume: every 16th voxel in x and y on
    every 32nd slice (the oracle filters every detector row by FFT)."""
    rg, ig, plan, proj, img = cbct_flat_512
    g = dict(kind="flat", offset_s=0.0, offset_t=0.0, orbit_start=0.0, source_offset=0.0, **GEOM3)
    p = proj.cpu().numpy().astype(np.float64)
    filt = O.sino_filter_fft(p * O.fdk_weights(g), O.fbp_filter(g), workers=_workers())
    # voxel centres d (i - (n-1)/2) at i = 0, 16, ... (x, y) and 0, 32, ... (z): a coarser grid
    # with the same centres, offset (stride - 1) / (2 stride) voxels of its own size
    sub = dict(dims=(32, 32, 8), deltas=(8.0, 8.0, 16.0), offsets=(15 / 32, 15 / 32, 31 / 64))
    return O.cbct_back(filt, g, sub)


def _sample(img):
    return img.cpu().numpy()[0:256:32, 0:512:16, 0:512:16]


def test_cbct_flat_512_sampled_voxels_match_fp64_oracle(cbct_flat_512, cbct_flat_512_ref):
    ref = cbct_flat_512_ref
    got = _sample(cbct_flat_512[4])
    assert got.shape == ref.shape
    assert O.rel_rmse(got, ref) < 1e-5
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


def test_cbct_flat_512_f16_form_meets_1e4(cbct_flat_512, cbct_flat_512_ref):
    """The F16 storage form (FP16 quads of the filtered projections, FP32 accumulation) on the
    benchmark workload: relative RMSE <= 1e-4 against the FP64 oracle, the accuracy bound the
    benchmark's metric states for a reduced-precision form, and max error <= 2e-4 max|ref|."""
    rg, ig, plan, proj, img = cbct_flat_512
    p16 = S.plan_fbp(rg, ig, storage="f16")
    assert p16.info()["f16_quads"] and p16.info()["sample_bytes"] == 8
    got = _sample(S.fdk(p16, proj))
    ref = cbct_flat_512_ref
    assert O.rel_rmse(got, ref) <= 1e-4
    assert np.abs(got - ref).max() <= 2e-4 * np.abs(ref).max()


def test_cbct_flat_512_scaling_is_exact_and_sums_add(cbct_flat_512):
    import torch
    rg, ig, plan, proj, img = cbct_flat_512
    twice = S.fdk(plan, 2 * proj)
    assert torch.equal(twice, 2 * img)  # every rounding commutes with scaling by 2
    other = S.ellipsoid_proj(rg, S.random_ellipsoids(12, 33, 100.0, 50.0), device=True)
    both = S.fdk(plan, proj + other)
    parts = img + S.fdk(plan, other)
    rel = float((both - parts).pow(2).sum().sqrt() / parts.pow(2).sum().sqrt())
    assert rel < 1e-6


def test_par_256x180_hann_full_size(cuda):
    g = dict(kind="par", nb=256, d=1.0, offset=0.0, na=180, orbit=180.0, orbit_start=0.0)
    igd = dict(dims=(256, 256), deltas=(1.0, 1.0))
    ell = S.random_ellipses(10, 1, 100.0)
    sino = O.ellipse_sino(g, ell).astype(np.float32)
    ref = O.fbp(g, igd, sino, shape="hann")
    rg = S.SinoPar(nb=256, d=1.0, na=180, orbit=180.0)
    out = S.fbp(S.plan_fbp(rg, S.ImageGeom((256, 256), (1.0, 1.0)), window=S.Window("hann")), sino)
    # Inside the reconstruction FOV.  The image corners lie outside it and sit exactly on the
    # detector edge for axis-aligned views (at 90 deg the corner's bin is 1 - 7.8e-15 in FP64,
    # exactly 1 in FP32), so the whole-tap rule keeps or drops that tap depending on rounding.
    inside = np.asarray(S.ImageGeom((256, 256), (1.0, 1.0)).circle(S._rfov(rg) - 1.0))
    assert O.rel_rmse(out[inside], ref[inside]) < 1e-5
    assert np.abs(out - ref)[inside].max() <= 1e-4 * np.abs(ref).max()


def test_fan_arc_888x512_short_scan_noisy_full_size(cuda):
    base = dict(kind="arc", nb=888, d=1.0239, offset=0.0, dsd=949.075, dod=408.075, source_offset=0.0,
                orbit_start=0.0)
    orbit = 180 + 2 * math.degrees(float(np.max(np.abs(O.gamma(dict(base, na=2, orbit=360.0))))))
    g = dict(base, na=512, orbit=orbit)
    igd = dict(dims=(512, 512), deltas=(0.9766, 0.9766))
    ell = S.random_ellipses(20, 2, 220.0, axes=(4.0, 120.0), dens=(-0.3, 1.0))
    sino = O.ellipse_sino(g, ell)
    sino = (sino + 0.005 * np.abs(sino).max() * np.random.default_rng(102).standard_normal(sino.shape))
    sino = sino.astype(np.float32)
    ref = O.fbp(g, igd, sino)
    rg = S.SinoFanArc(nb=888, d=1.0239, dsd=949.075, dod=408.075, na=512, orbit=orbit)
    ig = S.ImageGeom((512, 512), (0.9766, 0.9766))
    out = S.fbp(S.plan_fbp(rg, ig), sino)
    # Inside the FOV (rfov = dso sin(gamma_max) = 249 mm; the corners reach 353 mm and meet the
    # detector edges, where FP32 and FP64 rounding decide the whole-tap rule differently).
    # The white noise (0.5% of the peak) makes adjacent filtered bins differ by about the
    # signal itself, so the FP32 tap position (atan2 of the arc, ~1e-4 bin) shows through far
    # more than on smooth data: measured 2.7e-5, held to the stated 1e-4 FP32-vs-FP64 bar.
    inside = np.asarray(ig.circle(S._rfov(rg) - 1.0))
    err = O.rel_rmse(out[inside], ref[inside])
    assert err < 1e-4, (err, O.rel_rmse(out, ref))
    assert np.abs(out - ref)[inside].max() <= 1e-4 * np.abs(ref).max()
