"""GPU parity of the separable-footprint projector pair against the FP64 oracle (oracle.c
orc_sf_project / orc_sf_back, itself pinned in test_sf_cpu.py), its adjointness and determinism,
and its call paths.

Tolerances (FP32 footprints and sums against FP64): relative RMSE <= 1e-5 and max abs error
<= 1e-4 * max|ref|; adjointness <Ax, y> = <x, A'y> to 2e-6 relative (the same FP32 elements,
summed in different orders)."""
import math

import numpy as np
import pytest

import cases as C
import oracle as O
import sinograms as S

pytestmark = pytest.mark.gpu
RTOL_RMSE = 1e-5
MAX_REL = 1e-4


def close(x, ref, rmse=RTOL_RMSE, maxrel=MAX_REL):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    assert x.shape == ref.shape, (x.shape, ref.shape)
    e = O.rel_rmse(x, ref)
    m = np.abs(x - ref).max() / np.abs(ref).max()
    assert e <= rmse and m <= maxrel, f"rel_rmse={e:.3g} max_rel={m:.3g}"
    return e


def geom(kind, **kw):
    g = dict(kind=kind, nb=71, d=1.1, offset=0.25, na=33, orbit=360.0, orbit_start=7.0)
    if kind != "par":
        g.update(dsd=300.0, dod=140.0, source_offset=1.5)
    g.update(kw)
    return g


# the learned-filter / distance-driven workload: SinoFanArc 888 x 90 over 360 deg, 512^2 at 0.9766 mm
ARC888 = dict(kind="arc", nb=888, d=1.0239, offset=1.25, na=90, orbit=360.0, orbit_start=0.0, dsd=949.075,
              dod=408.075, source_offset=0.0)
IG512 = dict(dims=(512, 512), deltas=(0.9766, 0.9766), offsets=(0.0, 0.0))

CASES = {
    "par": (geom("par"), dict(dims=(37, 29), deltas=(1.3, 0.9), offsets=(0.5, -1.25))),
    "arc": (geom("arc"), dict(dims=(37, 29), deltas=(1.3, 0.9), offsets=(0.5, -1.25))),
    "flat": (geom("flat"), dict(dims=(37, 29), deltas=(1.3, 0.9), offsets=(0.5, -1.25))),
    "par-180-neg-dy": (geom("par", orbit=180.0, orbit_start=0.0, na=20), dict(dims=(40, 33), deltas=(1.0, -1.0),
                                                                              offsets=(0.0, 0.0))),
    "flat-wide": (geom("flat", nb=301, d=1.0, offset=0.0, dsd=120.0, dod=50.0, na=40),
                  dict(dims=(48, 48), deltas=(1.0, 1.0), offsets=(0.0, 0.0))),
    "arc-wide": (geom("arc", nb=301, d=1.0, offset=0.0, dsd=120.0, dod=50.0, na=40),
                 dict(dims=(48, 48), deltas=(1.0, 1.0), offsets=(0.0, 0.0))),
}


def _run(g, ig, x, forward):
    plan = S.SFPlan(C.to_geom(g), C.to_image(ig, ig.get("mask")))
    return plan.project(x.astype(np.float32)) if forward else plan.backproject(x.astype(np.float32))


@pytest.mark.parametrize("name", list(CASES))
def test_sf_pair_matches_oracle(cuda, name):
    g, ig = CASES[name]
    rng = np.random.default_rng(11)
    nx, ny = ig["dims"]
    img = rng.random((ny, nx))
    sino = rng.random((g["na"], g["nb"]))
    close(_run(g, ig, img, True), O.sf_project(g, ig, img))
    close(_run(g, ig, sino, False), O.sf_back(g, ig, sino))


@pytest.mark.parametrize("kind", ["par", "arc", "flat"])
def test_sf_golden_fixtures(cuda, kind):
    """The committed FP64 fixtures (tests/golden/sf.npz) for the three geometries."""
    import os
    f = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sf.npz"))
    c = C.SF[kind]
    close(_run(c["rg"], c["ig"], f[f"{kind}_image"], True), f[f"{kind}_ref_proj"])
    close(_run(c["rg"], c["ig"], f[f"{kind}_sino"], False), f[f"{kind}_ref_back"])


@pytest.mark.parametrize("kind", ["par", "arc", "flat"])
def test_sf_masked_image(cuda, kind):
    g, ig = CASES[kind]
    nx, ny = ig["dims"]
    mask = np.random.default_rng(2).random((ny, nx)) > 0.3
    igm = dict(ig, mask=mask)
    img = np.random.default_rng(3).random((ny, nx))
    close(_run(g, igm, img, True), O.sf_project(g, igm, img))
    sino = np.random.default_rng(4).random((g["na"], g["nb"]))
    back = _run(g, igm, sino, False)
    close(back, O.sf_back(g, igm, sino))
    assert np.all(back[~mask] == 0)


def test_sf_full_size_arc888_matches_oracle(cuda):
    """The SinoFanArc 888 x 90, 512^2 workload of the distance-driven pair and the learned filter, on
    one of its seeded random-ellipse phantoms."""
    from sinograms import learned as L
    img = np.asarray(L.ellipse_image(C.to_image(IG512), L.phantom_ellipses(3), sub=2, device=False), np.float64)
    got = _run(ARC888, IG512, img, True)
    close(got, O.sf_project(ARC888, IG512, img))
    sino = np.asarray(got, np.float64)
    close(_run(ARC888, IG512, sino, False), O.sf_back(ARC888, IG512, sino))


@pytest.mark.parametrize("name", ["par", "arc", "flat", "arc-wide"])
def test_sf_pair_is_adjoint_on_the_gpu(cuda, name):
    g, ig = CASES[name]
    nx, ny = ig["dims"]
    rng = np.random.default_rng(5)
    x = rng.random((ny, nx)).astype(np.float32)
    y = rng.random((g["na"], g["nb"])).astype(np.float32)
    plan = S.SFPlan(C.to_geom(g), C.to_image(ig))
    lhs = float((plan.project(x).astype(np.float64) * y).sum())
    rhs = float((x.astype(np.float64) * plan.backproject(y)).sum())
    assert abs(lhs - rhs) <= 2e-6 * abs(lhs)


def test_sf_is_deterministic_and_paths_agree(cuda):
    import torch
    g, ig = ARC888, IG512
    plan = S.SFPlan(C.to_geom(g), C.to_image(ig))
    img = np.random.default_rng(8).random((512, 512)).astype(np.float32)
    a = plan.project(img)
    np.testing.assert_array_equal(a, plan.project(img))                      # bit-identical reruns
    np.testing.assert_array_equal(a, S.project_sf(C.to_geom(g), C.to_image(ig), img))  # one-shot form
    d = plan.project(torch.from_numpy(img).to(cuda))                         # device pointers
    np.testing.assert_array_equal(a, d.cpu().numpy())
    out = torch.empty((g["na"], g["nb"]), device=cuda)
    plan.project(torch.from_numpy(img).to(cuda), out=out, sync=False)        # asynchronous
    torch.cuda.synchronize()
    np.testing.assert_array_equal(a, out.cpu().numpy())
    b = plan.backproject(a)
    np.testing.assert_array_equal(b, plan.backproject(a))
    np.testing.assert_array_equal(b, S.backproject_sf(C.to_geom(g), C.to_image(ig), a))
    np.testing.assert_array_equal(b, plan.backproject(torch.from_numpy(a).to(cuda)).cpu().numpy())


@pytest.mark.parametrize("splits", [1, 2, 3, 8, 64])
def test_sf_forward_line_splits(cuda, splits):
    """Any split of the image lines over thread blocks gives the oracle's projection; each split
    count is deterministic."""
    for name in ("arc", "flat-wide", "par-180-neg-dy"):
        g, ig = CASES[name]
        nx, ny = ig["dims"]
        img = np.random.default_rng(12).random((ny, nx)).astype(np.float32)
        plan = S.SFPlan(C.to_geom(g), C.to_image(ig))
        plan.line_splits = splits
        assert plan.line_splits == splits
        a = plan.project(img)
        close(a, O.sf_project(g, ig, img))
        np.testing.assert_array_equal(a, plan.project(img))
    with pytest.raises(S.SinogramsArgumentError):
        plan.line_splits = 0


def test_sf_parallel_single_pixels_are_box_splines(cuda):
    """SinoPar on the GPU: one pixel's projection is the bin-integrated Radon transform of the
    rectangle, zwart_powell(k - uc, (dx cos/ds, dy sin/ds, 1, 0)) dx dy / ds (zwart_powell.jl:23-58)."""
    g = dict(kind="par", nb=40, d=0.45, offset=0.1, na=12, orbit=180.0, orbit_start=0.0)
    dx, dy = 1.0, 0.7
    ig = dict(dims=(5, 4), deltas=(dx, dy), offsets=(0.3, -0.2))
    img = np.zeros((4, 5), np.float32)
    img[2, 3] = 1.0
    got = _run(g, ig, img, True)
    wb = (g["nb"] - 1) / 2 + float(np.float32(g["offset"]))
    xc, yc = dx * (3 - 2 - 0.3), dy * (2 - 1.5 + 0.2)
    for v, b in enumerate(O.ar(g)):
        uc = (xc * math.cos(b) + yc * math.sin(b)) / g["d"] + wb
        z = (dx * math.cos(b) / g["d"], dy * math.sin(b) / g["d"], 1.0, 0.0)
        ref = O.zwart_powell_z(np.arange(g["nb"]) - uc, z) * dx * dy / g["d"]
        assert np.abs(got[v] - ref).max() <= 2e-5 * ref.max()


@pytest.mark.parametrize("case", [
    (dict(kind="par", nb=1, d=1.0, offset=0.0, na=1, orbit=180.0, orbit_start=0.0), dict(dims=(1, 1), deltas=(2.0, 2.0))),
    (dict(kind="arc", nb=3, d=1.0, offset=0.4, na=2, orbit=360.0, orbit_start=0.0, dsd=50.0, dod=20.0,
          source_offset=0.0), dict(dims=(3, 2), deltas=(1.0, 1.0))),
    # detector narrower than the image: bins outside 0..nb-1 are dropped
    (dict(kind="flat", nb=9, d=1.0, offset=-3.0, na=7, orbit=360.0, orbit_start=45.0, dsd=200.0, dod=100.0,
          source_offset=0.0), dict(dims=(30, 30), deltas=(1.0, 1.0))),
    # views at exactly 0, 45, 90, ... degrees (degenerate trapezoids: boxes and triangles)
    (dict(kind="par", nb=50, d=0.5, offset=0.0, na=8, orbit=360.0, orbit_start=0.0), dict(dims=(16, 16), deltas=(1.0, 1.0))),
    (dict(kind="flat", nb=50, d=1.0, offset=0.0, na=8, orbit=360.0, orbit_start=0.0, dsd=200.0, dod=100.0,
          source_offset=0.0), dict(dims=(16, 16), deltas=(1.0, 1.0))),
], ids=["1x1", "tiny-arc", "narrow-detector", "par-axes", "flat-axes"])
def test_sf_edge_cases(cuda, case):
    g, ig = case
    ig = dict(ig, offsets=(0.0, 0.0))
    nx, ny = ig["dims"]
    rng = np.random.default_rng(6)
    img = rng.random((ny, nx))
    sino = rng.random((g["na"], g["nb"]))
    close(_run(g, ig, img, True), O.sf_project(g, ig, img))
    close(_run(g, ig, sino, False), O.sf_back(g, ig, sino))


@pytest.mark.parametrize("kind", ["par", "arc", "flat"])
@pytest.mark.parametrize("scale", ["fine-pixels", "fine-bins"])
def test_sf_extreme_pixel_to_bin_ratios(cuda, kind, scale):
    """fine-pixels: 0.25 mm pixels under 4 mm bins, so a 256-bin chunk of the forward projector sees
    more footprints per image line than one shared-memory pass holds (several passes per line);
    fine-bins: 4 mm pixels over 0.1 mm bins, so every footprint spans tens of bins."""
    if scale == "fine-pixels":
        g = geom(kind, nb=300, d=4.0, offset=0.5, na=12)
        ig = dict(dims=(1024, 48), deltas=(0.25, 0.3), offsets=(0.0, 3.0))
    else:
        g = geom(kind, nb=900, d=0.1, offset=-0.5, na=12)
        ig = dict(dims=(20, 18), deltas=(4.0, 3.5), offsets=(0.25, 0.0))
    if kind != "par":
        g.update(dsd=900.0, dod=400.0)
    nx, ny = ig["dims"]
    rng = np.random.default_rng(21)
    img = rng.random((ny, nx))
    sino = rng.random((g["na"], g["nb"]))
    for splits in (1, 3):
        plan = S.SFPlan(C.to_geom(g), C.to_image(ig))
        plan.line_splits = splits
        close(plan.project(img.astype(np.float32)), O.sf_project(g, ig, img))
    close(_run(g, ig, sino, False), O.sf_back(g, ig, sino))


def test_sf_large_image_matches_oracle(cuda):
    """A 1024^2 image at 0.5 mm under the 888-bin flat detector, 60 views."""
    g = dict(ARC888, kind="flat", na=60, orbit_start=3.0, offset=-0.75)
    ig = dict(dims=(1024, 1024), deltas=(0.5, 0.5), offsets=(0.0, 0.0))
    img = np.random.default_rng(22).random((1024, 1024))
    close(_run(g, ig, img, True), O.sf_project(g, ig, img))


def test_sf_and_dd_agree_with_the_analytic_sinogram(cuda):
    """On the 888 x 90 arc scan (centred detector, as the distance-driven pair has no offset) both
    system models approach the analytic line integrals of an ellipse phantom; SF is the closer one."""
    import torch
    from sinograms import learned as L
    g = dict(ARC888, offset=0.0)
    rg, ig = C.to_geom(g), C.to_image(IG512)
    ell = np.array([[20.0, -15.0, 120.0, 80.0, 0.5, 1.0], [-40.0, 30.0, 40.0, 60.0, -0.3, 0.5]])
    img = L.ellipse_image(ig, ell, sub=4, device=False)
    ref = O.ellipse_sino(g, ell)
    e_sf = O.rel_rmse(_run(g, IG512, img, True), ref)
    dd = L.dd_project(torch.from_numpy(img).to(cuda), S.BddGeo.from_geoms(rg, ig)).cpu().numpy()
    e_dd = O.rel_rmse(dd, ref)
    assert e_sf < 1e-2, (e_sf, e_dd)
    assert e_sf < e_dd, (e_sf, e_dd)


def _random_case(seed):
    """A seeded random geometry inside the pair's limits: the image within 0.99 dso, arc detectors
    narrower than +-90 degrees."""
    rng = np.random.default_rng(1000 + seed)
    kind = ("par", "arc", "flat")[seed % 3]
    nx, ny = int(rng.integers(1, 48)), int(rng.integers(1, 48))
    dx, dy = float(rng.uniform(0.3, 2.5)), float(rng.uniform(0.3, 2.5)) * (1 if rng.random() < 0.8 else -1)
    ig = dict(dims=(nx, ny), deltas=(dx, dy), offsets=(float(rng.uniform(-2, 2)), float(rng.uniform(-2, 2))))
    g = dict(kind=kind, nb=int(rng.integers(1, 160)), d=float(rng.uniform(0.2, 3.0)),
             offset=float(np.float32(rng.uniform(-3, 3))), na=int(rng.integers(1, 40)),
             orbit=float(rng.choice([180.0, 360.0, 217.5])), orbit_start=float(rng.uniform(-90, 90)))
    if kind != "par":
        rmax = np.hypot(abs(dx) * (nx / 2 + 2), abs(dy) * (ny / 2 + 2))
        dso = float(rmax / 0.9 + rng.uniform(5, 300))
        dsd = dso + float(rng.uniform(10, 400))
        # keep the arc detector inside +-80 degrees
        if kind == "arc":
            g["nb"] = min(g["nb"], int(2 * 1.39 * dsd / g["d"]) - 2)
        g.update(dsd=dsd, dod=dsd - dso, source_offset=float(rng.uniform(-3, 3)))
    return g, ig


@pytest.mark.parametrize("seed", range(18))
def test_sf_random_geometries(cuda, seed):
    g, ig = _random_case(seed)
    nx, ny = ig["dims"]
    rng = np.random.default_rng(seed)
    img = rng.random((ny, nx))
    sino = rng.random((g["na"], g["nb"]))
    ref_p = O.sf_project(g, ig, img)
    ref_b = O.sf_back(g, ig, sino)
    if np.abs(ref_p).max() > 0:  # the image may miss a narrow detector entirely
        close(_run(g, ig, img, True), ref_p)
    else:
        assert np.abs(_run(g, ig, img, True)).max() == 0
    if np.abs(ref_b).max() > 0:
        close(_run(g, ig, sino, False), ref_b)
    else:
        assert np.abs(_run(g, ig, sino, False)).max() == 0
