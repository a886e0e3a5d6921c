"""The 2D back-projector's per-view forms against the FP64 oracle (fbp_back,
back-par.jl:184-203 / back-fan.jl:11-32).

The kernel classifies each (32 x 32 pixel tile, view) pair from the tile's corners: fast (every tap
valid and staged in shared memory), checked (staged, per-pixel tap rule), global (tile not wholly in
front of the source: taps from global memory) and none (tile off the detector).  These geometries
make every form occur, use an arc detector wide enough for the atan2 fallback, and split a prime
number of views over a cluster."""
import numpy as np
import pytest

import oracle as O
import sinograms as S

import cases as C

pytestmark = pytest.mark.gpu


def _err(x, ref):
    x = np.asarray(x, np.float64)
    return O.rel_rmse(x, ref), np.abs(x - ref).max() / np.abs(ref).max()


def _check(rg, ig, seed, ia_skip=1, ring=None):
    """Relative RMSE <= 1e-5 and max error <= 1e-4 max|ref| against FP64, or, where single precision
    itself is ill-conditioned, within 2x of the distance of the oracle's own FP32 build.  With
    `ring` = (dso, w) the bar applies outside |rho - dso| <= w: pixels passing close to the source
    have d = dso + x sin - y cos and r both near 0 for some view, and w2 = (dsd/d)^2 turns their
    rounding into arbitrary values in any FP32 arithmetic; the whole image is held to 4x."""
    s = np.random.default_rng(seed).standard_normal((rg["na"], rg["nb"])).astype(np.float32)
    ref = O.fbp_back(rg, ig, s, ia_skip=ia_skip)
    r32 = O.fbp_back(rg, ig, s, ia_skip=ia_skip, bits=32)
    out = np.asarray(S.fbp_back(C.to_geom(rg), C.to_image(ig), s, ia_skip=ia_skip), np.float64)
    keep = np.ones(ref.shape, bool)
    if ring is not None:
        ax = O.image_axes(ig)
        keep = np.abs(np.hypot(ax[0][None, :], ax[1][:, None]) - ring[0]) > ring[1]
        ew, mw = _err(out, ref)
        ew32, mw32 = _err(r32, ref)
        assert ew <= 4 * ew32 and mw <= 4 * mw32, f"whole image: {ew:.3g} {mw:.3g} (FP32 oracle {ew32:.3g} {mw32:.3g})"
    e32, m32 = _err(r32[keep], ref[keep])
    e, m = _err(out[keep], ref[keep])
    assert e <= max(1e-5, 2 * e32) and m <= max(1e-4, 2 * m32), (
        f"rel_rmse={e:.3g} max_rel={m:.3g} (FP32 oracle: {e32:.3g}, {m32:.3g})")


@pytest.mark.parametrize("kind", ["flat", "arc"])
def test_fan_image_wider_than_the_source_circle(cuda, kind):
    # dso = 40 mm, image half-width 48 mm: tiles straddle and lie behind the source (global form),
    # tiles beside the fan miss the detector (none), the rest are fast or checked
    rg = dict(kind=kind, nb=64, d=1.0, offset=0.0, na=40, orbit=360.0, orbit_start=0.0, source_offset=0.0,
              dsd=60.0, dod=20.0)
    _check(rg, dict(dims=(96, 96), deltas=(1.0, 1.0)), seed=11, ring=(40.0, 6.0))


def test_arc_detector_wider_than_45_degrees_uses_atan2(cuda):
    # fan half-angle (48.5 + 4) / 40 = 1.31 rad: outside the angle polynomial's range
    rg = dict(kind="arc", nb=96, d=1.0, offset=0.75, na=36, orbit=360.0, orbit_start=5.0, source_offset=0.0,
              dsd=40.0, dod=10.0)
    _check(rg, dict(dims=(48, 40), deltas=(0.8, 0.8), offsets=(0.25, -0.5)), seed=12)


@pytest.mark.parametrize("ia_skip", [1, 2])
def test_par_offset_detector_prime_views(cuda, ia_skip):
    # detector shifted by 10.5 bins: many tiles partly or wholly off it (checked / none); 37 views
    # split unevenly over the cluster
    rg = dict(kind="par", nb=100, d=1.0, offset=10.5, na=37, orbit=180.0, orbit_start=3.0)
    _check(rg, dict(dims=(128, 96), deltas=(1.0, 1.0)), seed=13, ia_skip=ia_skip)


def test_flat_source_offset_and_many_views(cuda):
    # source_offset moves the rays' centre (back-fan.jl:303); 300 views use several view chunks
    rg = dict(kind="flat", nb=120, d=0.9, offset=-2.25, na=300, orbit=360.0, orbit_start=0.0, source_offset=1.5,
              dsd=200.0, dod=80.0)
    _check(rg, dict(dims=(70, 66), deltas=(1.1, 1.2)), seed=14)
