"""GPU parity: every CUDA entry point against the FP64 oracle (committed fixtures and live
oracle runs on the same seeded inputs), plus the reference's conservation tests run on
the GPU path.

Tolerances (FP32 arithmetic against FP64): relative RMSE <= 1e-5 and max abs error
<= 1e-4 * max|ref| for the FP32 forms; the reduced-precision storage forms (F16 quads, BF16)
follow `form_bars`."""
import math
import os

import numpy as np
import pytest

import cases as C
import oracle as O
import sinograms as S

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
RTOL_RMSE = 1e-5
MAX_REL = 1e-4


form_bars = C.form_bars


def fix(name):
    return np.load(os.path.join(HERE, "golden", f"{name}.npz"))


def close(x, ref, rmse=RTOL_RMSE, maxrel=MAX_REL):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    assert x.shape == ref.shape, (x.shape, ref.shape)
    e = O.rel_rmse(x, ref)
    m = np.abs(x - ref).max() / np.abs(ref).max()
    assert e <= rmse and m <= maxrel, f"rel_rmse={e:.3g} max_rel={m:.3g}"
    return e


def test_fdk_flat_fixture(cuda):
    f, c = fix("fdk_flat"), C.FDK_FLAT
    plan = S.plan_fbp(C.to_geom(c["rg"]), C.to_image(c["ig"]), window=S.Window(c["window"]))
    assert plan.info()["tma"], plan.info()
    close(S.fdk(plan, f["proj"]), f["ref"])


@pytest.mark.parametrize("kind", ["arc", "flat"])
@pytest.mark.parametrize("storage", ["f32", "bf16", "f16"])
def test_fdk_ragged_sizes(cuda, kind, storage):
    """ns not a multiple of the TMA alignment, partial voxel tiles in x, y and z."""
    rg = C.ct(kind, ns=37, nt=23, na=19, offset_s=-0.25, offset_t=0.5, dsd=150.0, dod=50.0)
    ig = dict(dims=(19, 21, 13), deltas=(0.9, 1.0, 1.1), offsets=(0.3, 0.0, -0.2))
    proj = O.ellipsoid_proj(rg, C.ELL3).astype(np.float32)
    ref = O.fdk(rg, ig, proj)
    plan = S.plan_fbp(C.to_geom(rg), C.to_image(ig), storage=storage)
    assert plan.info()["tma"] and plan.info()["pitch"] == 40
    assert plan.info()["f16_quads"] == (storage == "f16")
    close(S.fdk(plan, proj), ref, *form_bars(storage, rg["na"]))


def test_fdk_helix_default_ignores_source_z(cuda):
    """A CtSourceHelix scan reconstructs exactly like its circular twin unless asked
    (the reference's cbct_back ignores source z, cbct-back.jl:188-189)."""
    c = C.HELIX
    circ = {k: v for k, v in c["rg"].items() if k not in ("src", "pitch", "source_z0")}
    proj = O.ellipsoid_proj(circ, C.ELL3).astype(np.float32)
    a = S.fdk(S.plan_fbp(C.to_geom(c["rg"]), C.to_image(c["ig"])), proj)
    b = S.fdk(S.plan_fbp(C.to_geom(circ), C.to_image(c["ig"])), proj)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("storage", ["f32", "bf16", "f16"])
def test_fdk_helix_source_z(cuda, storage):
    """source_z=True: t' = mag * (z - source_zs[view]) in the TMA back-projector (box
    pre-pass and producer use the shifted z) against the oracle."""
    c = C.HELIX
    proj = O.ellipsoid_proj(c["rg"], C.ELL3).astype(np.float32)
    ref = O.fdk(c["rg"], c["ig"], proj, source_z=True)
    plan = S.plan_fbp(C.to_geom(c["rg"]), C.to_image(c["ig"]), storage=storage, source_z=True)
    assert plan.info()["tma"]
    out = S.fdk(plan, proj)
    close(out, ref, *form_bars(storage, c["rg"]["na"]))
    assert O.rel_rmse(out, O.fdk(c["rg"], c["ig"], proj)) > 1e-2  # the shift matters here


def test_fdk_arc_short_fixture_mask_window(cuda):
    f, c = fix("fdk_arc_short"), C.FDK_ARC_SHORT
    mask = C.cyl_mask(c["ig"], c["mask_r"])
    plan = S.plan_fbp(C.to_geom(c["rg"]), C.to_image(c["ig"], mask), window=S.Window(c["window"], c["cutoff"]))
    out = S.fdk(plan, f["proj"])
    close(out, f["ref"])
    assert np.all(out[~mask] == 0)


@pytest.mark.parametrize("name,case", [("fbp_par", C.PAR), ("fbp_arc_short", C.ARC_SHORT), ("fbp_flat", C.FLAT)])
def test_fbp_fixtures(cuda, name, case):
    f = fix(name)
    plan = S.plan_fbp(C.to_geom(case["rg"]), C.to_image(case["ig"]), window=S.Window(case["window"]))
    close(S.fbp(plan, f["sino"]), f["ref"])


def test_sino_filter_wrap_fixture(cuda):
    f = fix("sino_filter_wrap")
    close(S.fbp_sino_filter(f["x"], f["Hk"], extra=C.FILTER_WRAP["extra"]), f["ref"], maxrel=2e-4)


@pytest.mark.parametrize("nb,npad", [(64, 128), (100, 128), (512, 1024), (888, 1024), (37, 64)])
def test_sino_filter_random(cuda, nb, npad):
    rng = np.random.default_rng(nb)
    x = rng.standard_normal((9, 3, nb)).astype(np.float32)
    Hk = O.fbp_filter(dict(kind="flat", nb=nb, d=1.0), npad=npad, shape="hann")
    close(S.fbp_sino_filter(x, Hk), O.sino_filter(x, Hk), maxrel=2e-4)


def test_sino_filter_many_tiles_smooth_rows(cuda):
    """Persistent tensor-core filter over many 128-row tiles (both accumulators of every
    CTA in use), three 256-sample output blocks, and smooth rows on which the ramp filter
    cancels ~100x -- the case the split-BF16 GEMM on first differences is built for."""
    nb, npad, nrows = 520, 1024, 40000
    rng = np.random.default_rng(7)
    s = np.arange(nb)[None, :]
    c = rng.uniform(100, 420, (nrows, 1))
    w = rng.uniform(40, 90, (nrows, 1))
    x = np.sqrt(np.clip(w * w - (s - c) ** 2, 0, None)) * rng.uniform(0.5, 2.0, (nrows, 1))
    x = x.astype(np.float32)
    Hk = O.fbp_filter(dict(kind="flat", nb=nb, d=1.0), npad=npad)
    ref = O.sino_filter_fft(x.astype(np.float64), Hk)
    out = S.fbp_sino_filter(x, Hk, extra=5)
    assert out.shape == (nrows, nb + 5) and np.all(out[:, nb:] == 0)
    close(out[:, :nb], ref, rmse=1e-6, maxrel=1e-5)


def test_bdd_fixtures(cuda):
    f, g = fix("bdd"), C.BDD
    geo = S.BddGeo(g["DSD"], g["DS0"], g["pSize"], g["dSize"], g["nPix"], g["nDet"], g["angle"])
    close(S.project_bdd(f["phantom"], geo), f["ref_proj"])
    close(S.backproject_bdd(f["sino"], geo), f["ref_back"])


@pytest.mark.parametrize("kind", ["arc", "flat"])
@pytest.mark.parametrize("ia_skip", [1, 3])
def test_cbct_back_seam(cuda, kind, ia_skip):
    rg = C.ct(kind, ns=40, nt=30, na=25, offset_s=0.25)
    ig = dict(dims=(20, 18, 14), deltas=(1.0, 1.0, 1.3), offsets=(0.0, 0.5, -0.5))
    rng = np.random.default_rng(3)
    proj = rng.standard_normal((25, 30, 40)).astype(np.float32)
    mask = rng.random((14, 18, 20)) > 0.2
    ref = O.cbct_back(proj, rg, dict(ig, mask=mask), ia_skip=ia_skip)
    out = S.cbct_back(proj, C.to_geom(rg), C.to_image(ig, mask), ia_skip=ia_skip)
    close(out, ref)


@pytest.mark.parametrize("case", [C.PAR, C.ARC_SHORT, C.FLAT], ids=["par", "arc", "flat"])
def test_fbp_back_seam_ia_skip(cuda, case):
    rng = np.random.default_rng(5)
    rg = case["rg"]
    s = rng.standard_normal((rg["na"], rg["nb"])).astype(np.float32)
    ax = O.image_axes(case["ig"])
    mask = (ax[0][None, :] ** 2 + ax[1][:, None] ** 2) <= 4.0 ** 2
    for skip in (1, 2):
        ref = O.fbp_back(rg, dict(case["ig"], mask=mask), s, ia_skip=skip)
        out = S.fbp_back(C.to_geom(rg), C.to_image(case["ig"], mask), s, ia_skip=skip)
        close(out, ref)


def test_device_pointer_path_equals_host(cuda):
    import torch
    f, c = fix("fdk_flat"), C.FDK_FLAT
    plan = S.plan_fbp(C.to_geom(c["rg"]), C.to_image(c["ig"]))
    host = S.fdk(plan, f["proj"])
    dev = S.fdk(plan, torch.as_tensor(f["proj"], device="cuda"))
    assert isinstance(dev, torch.Tensor) and dev.is_cuda
    np.testing.assert_array_equal(dev.cpu().numpy(), host)


def test_fbp_stack_equals_slices(cuda):
    """fbp(plan, sino3) loops the 2D path over slices (fbp.jl:46-68); linearity x5
    as in test/fbp2/fbp-par.jl:45-49."""
    f, c = fix("fbp_par"), C.PAR
    plan = S.plan_fbp(C.to_geom(c["rg"]), C.to_image(c["ig"]), window=S.Window(c["window"]))
    one = S.fbp(plan, f["sino"])
    stack = S.fbp(plan, np.stack([f["sino"], 5 * f["sino"]]))
    np.testing.assert_allclose(stack[0], one, rtol=0, atol=0)
    np.testing.assert_allclose(stack[1], 5 * one, rtol=1e-5, atol=1e-6 * np.abs(one).max())


def test_phantom_projectors(cuda):
    g = C.ARC_SHORT["rg"]
    close(S.ellipse_sino(C.to_geom(g), C.ELL2), O.ellipse_sino(g, C.ELL2), rmse=1e-7, maxrel=1e-6)
    rg = C.FDK_FLAT["rg"]
    close(S.ellipsoid_proj(C.to_geom(rg), C.ELL3), O.ellipsoid_proj(rg, C.ELL3), rmse=1e-5, maxrel=1e-4)


# ------------------------------------------------ reference conservation tests on the GPU

def _disk_err(rec, dx):
    return abs(float(np.sum(rec, dtype=np.float64)) * dx * dx - math.pi * 4) / (math.pi * 4)


def test_gpu_fbp_par_conservation(cuda):
    nr, dr, na = 64, 10 / 64, 128  # test/fbp2/fbp-par.jl:12-33
    rg = S.SinoPar(nb=nr, d=dr, na=na)
    s = S.ellipse_sino(rg, [[2.0, 1.0, 2.0, 2.0, 0.0, 1.0]])
    assert _disk_err(S.fbp(s, dr=dr), dr) < 2e-4
    rg = S.SinoPar(d=0.1)  # :35-49
    ig = S.ImageGeom((128, 128), (0.1, 0.1))
    ig = ig.with_mask(ig.circle(S._rfov(rg)))
    s = S.ellipse_sino(rg, [[2.0, 1.0, 2.0, 2.0, 0.0, 1.0]])
    rec = S.fbp(S.plan_fbp(rg, ig), np.stack([s, 5 * s]))
    assert _disk_err(rec[0], 0.1) < 5e-4 and _disk_err(rec[1] / 5, 0.1) < 5e-4


@pytest.mark.parametrize("cls", [S.SinoFanArc, S.SinoFanFlat])
@pytest.mark.parametrize("short", [False, True])
def test_gpu_fbp_fan_conservation(cuda, cls, short):
    rg = cls.short(d=0.1) if short else cls(d=0.1)  # test/fbp2/fbp-fan.jl:13-40
    ig = S.ImageGeom((128, 128), (0.1, 0.1))
    ig = ig.with_mask(ig.circle(S._rfov(rg)))
    s = S.ellipse_sino(rg, [[2.0, 1.0, 2.0, 2.0, 0.0, 1.0]])
    assert _disk_err(S.fbp(S.plan_fbp(rg, ig), s), 0.1) < 3e-3


@pytest.mark.parametrize("cls", [S.CtFanArc, S.CtFanFlat])
@pytest.mark.parametrize("short", [False, True])
@pytest.mark.parametrize("storage", ["f32", "bf16", "f16"])
def test_gpu_fdk_conservation(cuda, cls, short, storage):
    kw = dict(ns=64, nt=40, ds=1.0, dt=1.2)  # test/fbp3/fdk.jl:14-33
    rg = cls.short(na=59, **kw) if short else cls(na=32, **kw)
    ig = S.ImageGeom((30, 28, 26), (1.0, 1.0, 1.0))
    proj = S.ellipsoid_proj(rg, [[2.0, 3.0, 4.0, 8.0, 7.0, 6.0, 0.0, 0.0, 0.0, 1.0]])
    rec = S.fdk(S.plan_fbp(rg, ig, storage=storage), proj)
    vt = 4 / 3 * math.pi * 8 * 7 * 6
    assert abs(float(rec.sum(dtype=np.float64)) - vt) / vt < (2e-2 if short else 3e-3)


def test_gpu_bdd_adjoint_and_shapes(cuda):
    rg = S.downsample(S.SinoFanFlat(nb=910, d=1.0239, na=360, dsd=949.0, dod=408.0), 4)  # test/sys2/bdd_2d.jl
    ig = S.ImageGeom((128, 128), (4.0, 4.0))
    geo = S.BddGeo.from_geoms(rg, ig)
    rng = np.random.default_rng(0)
    x = rng.random((128, 128)).astype(np.float32)
    y = rng.random((rg.nb, rg.na)).astype(np.float32)
    Ax, Aty = S.project_bdd(x, geo), S.backproject_bdd(y, geo)
    assert Ax.shape == (geo.nDet, len(geo.angle)) and Aty.shape == (128, 128)
    lhs, rhs = float(np.dot(Ax.ravel().astype(np.float64), y.ravel())), float(np.dot(x.ravel(), Aty.ravel()))
    assert lhs == pytest.approx(rhs, rel=2e-2)
    ogeo = O.bdd_geo(geo.DSD, geo.DS0, geo.pSize, geo.dSize, geo.nPix, geo.nDet, geo.angle)
    close(Ax, O.project_bdd(x, ogeo))
    close(Aty, O.backproject_bdd(y, ogeo))


def test_bdd_plan_matches_per_call_projector(cuda):
    """BddPlan (geometry kept on the GPU) gives the results of project_bdd / backproject_bdd,
    for host arrays and for device tensors with asynchronous calls.  Both run the same kernels;
    their partial sums meet in float atomics, so the order (and the last bits) may differ."""
    import torch
    f, g = fix("bdd"), C.BDD
    geo = S.BddGeo(g["DSD"], g["DS0"], g["pSize"], g["dSize"], g["nPix"], g["nDet"], g["angle"])
    plan = S.BddPlan(geo)
    ph, sino = f["phantom"].astype(np.float32), f["sino"].astype(np.float32)
    ref_p, ref_b = S.project_bdd(ph, geo), S.backproject_bdd(sino, geo)
    close(plan.project(ph), ref_p, rmse=1e-6, maxrel=1e-6)
    close(plan.backproject(sino), ref_b, rmse=1e-6, maxrel=1e-6)
    for _ in range(2):  # repeated calls on the plan's scratch
        out_p = plan.project(torch.as_tensor(ph, device="cuda"), sync=False)
        out_b = plan.backproject(torch.as_tensor(sino, device="cuda"), sync=False)
        torch.cuda.synchronize()
        close(out_p.cpu().numpy(), ref_p, rmse=1e-6, maxrel=1e-6)
        close(out_b.cpu().numpy(), ref_b, rmse=1e-6, maxrel=1e-6)
    with pytest.raises(S.SinogramsArgumentError):
        plan.project(ph[:-1])


@pytest.mark.parametrize("arc", [False, True], ids=["flat", "arc"])
def test_bdd_pair_against_oracle_and_adjoint(cuda, arc):
    """The DD pair on a 90-view fan geometry against the FP64 oracle (flat: the reference's pair;
    arc: detector boundaries on the arc of radius DSD, the extension for SinoFanArc), per call and
    through a BddPlan; and the adjoint check of test/sys2/bdd_2d.jl:46-54 at its rtol 2e-2 (the
    first-view doubling of backproject_bdd keeps the pair from being exact adjoints)."""
    import torch
    rg = (S.SinoFanArc if arc else S.SinoFanFlat)(nb=222, d=4.0956, na=90, orbit=360.0, dsd=949.075, dod=408.075)
    ig = S.ImageGeom((128, 128), (3.9064, 3.9064))
    geo = S.BddGeo.from_geoms(rg, ig)
    assert geo.arc == arc
    ogeo = O.bdd_geo(geo.DSD, geo.DS0, geo.pSize, geo.dSize, geo.nPix, geo.nDet, geo.angle, arc=arc)
    rng = np.random.default_rng(21 + arc)
    x = rng.random((128, 128)).astype(np.float32)
    y = rng.random((rg.nb, rg.na)).astype(np.float32)
    Ax, Aty = S.project_bdd(x, geo), S.backproject_bdd(y, geo)
    close(Ax, O.project_bdd(x, ogeo))
    close(Aty, O.backproject_bdd(y, ogeo))
    plan = S.BddPlan(geo)
    close(plan.project(torch.as_tensor(x, device="cuda")).cpu().numpy(), Ax, rmse=1e-6, maxrel=1e-6)
    close(plan.backproject(torch.as_tensor(y, device="cuda")).cpu().numpy(), Aty, rmse=1e-6, maxrel=1e-6)
    lhs = float(np.dot(Ax.ravel().astype(np.float64), y.ravel()))
    rhs = float(np.dot(x.ravel().astype(np.float64), Aty.ravel()))
    assert lhs == pytest.approx(rhs, rel=2e-2)
    if arc:  # the arc geometry is not the flat one
        flat = S.BddGeo(geo.DSD, geo.DS0, geo.pSize, geo.dSize, geo.nPix, geo.nDet, geo.angle)
        assert O.rel_rmse(S.project_bdd(x, flat), Ax) > 1e-3


@pytest.mark.parametrize("npix,ndet", [(60, 40), (300, 1024), (300, 1025), (500, 2200)])
def test_bdd_project_bin_split_sizes(cuda, npix, ndet):
    """The projector splits the bins over the warps in groups of 32 (at most 4 per warp up to
    1024 bins, 8 up to 2048) and otherwise splits the rows: every split, warps without bins,
    the last group partial and image rows that do not fill the last block of 8, against the FP64
    oracle, per call and through a BddPlan.  Bins of 1.03 mm under 1 mm pixels (magnification
    1.75), the ratio of the reference's test geometry; the image's shadow spans several warps'
    bin ranges."""
    import torch
    angle = np.linspace(0.1, 2 * np.pi + 0.1, 12, endpoint=False)
    geo = S.BddGeo(949.0, 541.0, 1.0, 1.03, npix, ndet, angle)
    ogeo = O.bdd_geo(geo.DSD, geo.DS0, geo.pSize, geo.dSize, geo.nPix, geo.nDet, geo.angle)
    x = np.random.default_rng(ndet).random((npix, npix)).astype(np.float32)
    Ax = S.project_bdd(x, geo)
    close(Ax, O.project_bdd(x, ogeo))
    close(S.BddPlan(geo).project(torch.as_tensor(x, device="cuda")).cpu().numpy(), Ax, rmse=1e-6, maxrel=1e-6)


def test_bdd_oversized_image_is_an_argument_error(cuda):
    """The projection's shared-memory tiles bound nPix (2012 at nDet = 888): a larger image is
    refused with an argument error before any launch."""
    geo = S.BddGeo(949.0, 541.0, 0.25, 1.0239, 2100, 888, np.linspace(0, 2 * np.pi, 8, endpoint=False))
    with pytest.raises(S.SinogramsArgumentError):
        S.BddPlan(geo)


# -------------------------------------------------- reduced-precision storage forms

def test_fdk_storage_forms_error_level(cuda):
    """Each storage form against the FP64 oracle on a seeded random-ellipsoid phantom (the
    benchmark's phantom family and geometry, 180 views, reduced size), at the bars of
    `form_bars`.  The F16 form at the benchmark size itself: test_gpu_full_size.py."""
    rg = S.CtFanFlat(ns=128, nt=96, ds=1.0, dt=1.0, dsd=1000.0, dod=400.0, na=180)
    ig = S.ImageGeom((96, 96, 64), (1.0, 1.0, 1.0))
    ell = S.random_ellipsoids(30, 3, 25.0, 12.0, axes=(3.0, 20.0))
    proj = S.ellipsoid_proj(rg, ell)
    orc = dict(kind="flat", ns=128, nt=96, ds=1.0, dt=1.0, offset_s=0.0, offset_t=0.0, na=180, orbit=360.0,
               orbit_start=0.0, source_offset=0.0, dsd=1000.0, dod=400.0)
    ref = O.fdk(orc, dict(dims=(96, 96, 64), deltas=(1.0, 1.0, 1.0)), proj)
    for storage in ("f32", "f16", "bf16"):
        close(S.fdk(S.plan_fbp(rg, ig, storage=storage), proj), ref, *form_bars(storage, 180))


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
def test_fdk_power_of_two_scaling_is_exact(cuda, storage):
    """Scaling the projections by 2^k scales every stage exactly, including the F16 form's
    per-call FP16 scale (chosen from max|y|, so the stored quads do not change), far outside
    FP16's own range."""
    import torch
    c = C.FDK_FLAT
    proj = torch.as_tensor(O.ellipsoid_proj(c["rg"], C.ELL3).astype(np.float32), device="cuda")
    plan = S.plan_fbp(C.to_geom(c["rg"]), C.to_image(c["ig"]), storage=storage)
    base = S.fdk(plan, proj)
    for k in (-60, 40):
        assert torch.equal(S.fdk(plan, proj * 2.0 ** k), base * 2.0 ** k), k


@pytest.mark.parametrize("device", [False, True])
def test_zwart_powell_sino_gpu(cuda, device):
    """zwart_powell.(r, phi') of test/sys2/zwart_powell.jl:8-10 on the GPU (FP64) against the
    oracle restatement."""
    r = np.linspace(-1, 1, 101) * 2
    phi = np.linspace(0, np.pi, 181)
    out = S.zwart_powell_sino(r, phi, device=device)
    out = out.cpu().numpy() if device else out
    R, P = np.meshgrid(r, phi)
    np.testing.assert_allclose(out, O.zwart_powell(R, P), rtol=1e-9, atol=1e-12)
    assert out[90, 50] == pytest.approx(0.75, rel=1e-12)  # r = 0, phi = pi/2: the phi = 0 value by symmetry


@pytest.mark.parametrize("storage", ["f32", "bf16", "f16"])
def test_ctpar_fbp_against_oracle(cuda, storage):
    """CtPar (3D parallel beam; the reference defines it but does not reconstruct it):
    flat ramp, SinoPar's Parker x dbeta view weights, s = x cos + y sin, t = z."""
    c = C.CT_PAR
    rng = np.random.default_rng(11)
    g = c["rg"]
    proj = rng.standard_normal((g["na"], g["nt"], g["ns"])).astype(np.float32)
    ref = O.fdk(g, c["ig"], proj)
    plan = S.plan_fbp(C.to_geom(g), C.to_image(c["ig"]), storage=storage)
    # CtPar runs the direct back-projector, which has no FP16-quad form: F16 plans keep FP32
    assert not plan.info()["f16_quads"]
    # white-noise rows: the BF16 storage rounding (2^-9) shows through undamped, hence 4e-3
    close(S.fdk(plan, proj), ref, *((4e-3, 2e-2) if storage == "bf16" else (RTOL_RMSE, MAX_REL)))
    assert S.footprint_size(C.to_geom(g), C.to_image(c["ig"])) == pytest.approx(np.hypot(1.1, 1.0) / 1.0, rel=1e-6)


def test_ctpar_slices_equal_sinopar_fbp(cuda):
    """With the image z grid on the detector rows, a CtPar reconstruction's slice is the 2D
    SinoPar FBP (fbp.jl:24-68) of that detector row (t-lerp weight 0)."""
    # ds = dt keeps bt = z / ds + wt exact on the rows (an FP32 product could land just below
    # a row and drop it by the whole-tap rule)
    rg = S.CtPar(ns=48, nt=12, ds=1.0, dt=1.0, offset_s=0.25, offset_t=0.0, na=36, orbit=180.0)
    ig = S.ImageGeom((30, 26, 12), (0.7, 0.75, 1.0))
    rng = np.random.default_rng(5)
    proj = rng.standard_normal((rg.na, rg.nt, rg.ns)).astype(np.float32)
    vol = S.fdk(S.plan_fbp(rg, ig), proj)
    sp = S.SinoPar(nb=48, d=1.0, offset=0.25, na=36, orbit=180.0)
    plan2 = S.plan_fbp(sp, S.ImageGeom((30, 26), (0.7, 0.75)))
    for j in range(rg.nt - 1):  # the last row is dropped by the whole-tap rule 1 <= floor(bt) < nt
        close(vol[j], S.fbp(plan2, np.ascontiguousarray(proj[:, j, :])))
    assert np.all(vol[rg.nt - 1] == 0)


def test_bounded_wait_expires_with_an_error_status(cuda):
    """Failure detection without a GPU fault: a wait that nothing completes runs out of its
    (1 ms) budget, the call returns SGB_ERR_TIMEOUT with the message, and the context keeps
    working for the next reconstruction."""
    from sinograms import _lib
    st = _lib.lib().sgb_selftest_wait_timeout(2_000_000, None)
    assert st == _lib.SGB_ERR_TIMEOUT
    assert "bounded wait expired" in _lib.last_error()
    f, c = fix("fdk_flat"), C.FDK_FLAT
    plan = S.plan_fbp(C.to_geom(c["rg"]), C.to_image(c["ig"]), window=S.Window(c["window"]))
    close(S.fdk(plan, f["proj"]), f["ref"])


def test_async_host_plan_calls_match_blocking(cuda):
    """fdk / fbp with host buffers and sync=False enqueue the copies and kernels on the
    current stream; after plan.sync() the result equals the blocking call's."""
    import torch
    rng = np.random.default_rng(7)
    rg = S.CtFanFlat(ns=64, nt=32, ds=1.0, dt=1.0, dsd=500.0, dod=200.0, na=48)
    plan = S.plan_fbp(rg, S.ImageGeom((32, 32, 16), (1.0, 1.0, 1.0)))
    proj = rng.standard_normal((48, 32, 64)).astype(np.float32)
    ref = S.fdk(plan, proj)
    hp = torch.from_numpy(proj).pin_memory()
    out = torch.empty(ref.shape, dtype=torch.float32, pin_memory=True)
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        S.fdk(plan, hp.numpy(), out=out.numpy(), sync=False)
        plan.sync()
    assert np.array_equal(out.numpy(), ref)
    rg2 = S.SinoFanFlat(nb=96, d=1.0, na=60, orbit=360.0, dsd=400.0, dod=150.0)
    plan2 = S.plan_fbp(rg2, S.ImageGeom((48, 48), (1.5, 1.5)))
    sino = rng.standard_normal((60, 96)).astype(np.float32)
    ref2 = S.fbp(plan2, sino)
    hs = torch.from_numpy(sino).pin_memory()
    out2 = torch.empty(ref2.shape, dtype=torch.float32, pin_memory=True)
    with torch.cuda.stream(st):
        S.fbp(plan2, hs.numpy(), out=out2.numpy(), sync=False)
        plan2.sync()
    assert np.array_equal(out2.numpy(), ref2)


@pytest.mark.parametrize("passes", [2, 3])
def test_fdk_view_passes_agree(cuda, passes):
    """Views split over several launches (the later ones add to the volume) give the one-launch
    result to rounding and the oracle's."""
    f, c = fix("fdk_flat"), C.FDK_FLAT
    plan = S.plan_fbp(C.to_geom(c["rg"]), C.to_image(c["ig"]), window=S.Window(c["window"]))
    assert plan.info()["tma"], plan.info()
    plan.set_view_passes(1)
    one = S.fdk(plan, f["proj"])
    plan.set_view_passes(passes)
    assert plan.info()["view_passes"] == passes
    split = S.fdk(plan, f["proj"])
    assert O.rel_rmse(split, one) < 1e-6
    close(split, f["ref"])


def test_fdk_pair_boxes_too_large_fall_back_to_fp32_boxes(cuda):
    """A 16 x 16 x 16 voxel tile of 2 mm voxels at magnification up to ~1.9 needs a box of 128 x ~66
    samples: four pair (8-byte) stages exceed shared memory, four FP32 stages fit."""
    rg = C.ct("flat", ns=256, nt=128, ds=1.0, dt=1.0, na=48, dsd=300.0, dod=100.0)
    ig = dict(dims=(32, 32, 16), deltas=(2.0, 2.0, 2.0))
    proj = O.ellipsoid_proj(rg, C.ELL3).astype(np.float32)
    ref = O.fdk(rg, ig, proj)
    plan = S.plan_fbp(C.to_geom(rg), C.to_image(ig))
    info = plan.info()
    assert info["tma"] and info["sample_bytes"] == 4 and info["box"][0] == 128, info
    close(S.fdk(plan, proj), ref)
