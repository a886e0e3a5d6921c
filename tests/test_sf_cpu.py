"""Separable-footprint projector pair: the oracle pinned against the reference's own formulas, and
the library's host-side geometry (_tau, plan validation) -- no GPU needed.

Pins of the SF oracle (the reference has no SF projector; it has the pieces the model is built from):
  * _tau (src/geom/tau.jl:7-60): points on the rays of rays(rg) (sino-geom.jl:99-132) project to
    their own detector coordinate s/ds;
  * parallel beams: an SF element equals the box spline of the reference's zwart_powell(r, z) method
    (src/sys2/zwart_powell.jl:23-58) with directions (dx cos/ds, dy sin/ds, 1), times the pixel area
    over ds -- the exact bin-averaged Radon transform of the pixel;
  * footprint_size (src/sys2/footprint.jl:19-36) bounds the SF footprint widths (in bins) of the
    pixels inside the radial FOV it is computed from;
  * the pair is adjoint, conserves mass for parallel beams, and approaches the analytic line
    integrals of an ellipse for fan beams."""
import math

import numpy as np
import pytest

import cases as C
import oracle as O
import sinograms as S

KINDS = ["par", "arc", "flat"]


def geom(kind, **kw):
    g = dict(kind=kind, nb=71, d=1.1, offset=0.25, na=33, orbit=360.0, orbit_start=7.0)
    if kind != "par":
        g.update(dsd=300.0, dod=140.0, source_offset=1.5)
    g.update(kw)
    return g


IG = dict(dims=(37, 29), deltas=(1.3, 0.9), offsets=(0.5, -1.25))


@pytest.mark.parametrize("kind", KINDS)
def test_tau_points_on_rays_project_to_their_bin(kind):
    """tau.jl and sino-geom.jl:99-132 agree: a point on the ray (r, phi) of bin s has tau = s/ds."""
    g = geom(kind, source_offset=0.0)
    r, phi = O.sino_rays(g)
    s = O.s_axis(g)
    na, nb = r.shape
    for t in (-60.0, 0.0, 45.0):
        x = r * np.cos(phi) - t * np.sin(phi)
        y = r * np.sin(phi) + t * np.cos(phi)
        tau = O.tau(g, x.ravel(), y.ravel())
        got = np.array([tau[v, v * nb:(v + 1) * nb] for v in range(na)])
        np.testing.assert_allclose(got, np.broadcast_to(s / g["d"], got.shape), rtol=0, atol=1e-11)


@pytest.mark.parametrize("kind", KINDS)
def test_tau_library_matches_oracle(kind):
    g = geom(kind)
    rng = np.random.default_rng(3)
    x, y = rng.uniform(-40, 40, 50), rng.uniform(-40, 40, 50)
    got = S._tau(C.to_geom(g), x, y)
    np.testing.assert_allclose(got, O.tau(g, x, y), rtol=1e-13, atol=1e-12)
    assert got.shape == (g["na"], 50)


@pytest.mark.parametrize("deltas", [(1.0, 1.0), (1.0, 0.7), (0.6, 1.4)])
def test_sf_parallel_is_the_box_spline_of_zwart_powell(deltas):
    """SinoPar: the SF element of one pixel is zwart_powell(k - uc, (dx cos/ds, dy sin/ds, 1, 0)) *
    dx dy / ds, the bin-integrated Radon transform of the rectangle (zwart_powell.jl:23-58)."""
    ig = dict(dims=(5, 4), deltas=deltas, offsets=(0.3, -0.2))
    g = dict(kind="par", nb=40, d=0.45, offset=0.1, na=12, orbit=180.0, orbit_start=0.0)  # includes 0, 45, 90 deg
    img = np.zeros((4, 5))
    img[2, 3] = 1.0
    sino = O.sf_project(g, ig, img)
    dx, dy = deltas
    wb = (g["nb"] - 1) / 2 + float(np.float32(g["offset"]))
    xc, yc = dx * (3 - 2 - 0.3), dy * (2 - 1.5 + 0.2)
    for v, b in enumerate(O.ar(g)):
        uc = (xc * math.cos(b) + yc * math.sin(b)) / g["d"] + wb
        z = (dx * math.cos(b) / g["d"], dy * math.sin(b) / g["d"], 1.0, 0.0)
        ref = O.zwart_powell_z(np.arange(g["nb"]) - uc, z) * dx * dy / g["d"]
        np.testing.assert_allclose(sino[v], ref, rtol=0, atol=1e-12)


def test_sf_parallel_conserves_mass():
    g = dict(kind="par", nb=80, d=0.8, offset=-0.25, na=17, orbit=180.0, orbit_start=3.0)
    ig = dict(dims=(24, 20), deltas=(1.1, 0.9), offsets=(0.0, 0.0))
    img = np.random.default_rng(5).random((20, 24))
    sino = O.sf_project(g, ig, img)
    np.testing.assert_allclose(sino.sum(axis=1) * g["d"], img.sum() * 1.1 * 0.9, rtol=1e-12)


@pytest.mark.parametrize("kind", KINDS)
def test_sf_oracle_pair_is_adjoint(kind):
    g = geom(kind)
    ig = dict(IG, mask=np.random.default_rng(9).random((29, 37)) > 0.2)
    rng = np.random.default_rng(1)
    x, y = rng.random((29, 37)), rng.random((33, 71))
    lhs = (O.sf_project(g, ig, x) * y).sum()
    rhs = (x * O.sf_back(g, ig, y)).sum()
    assert lhs == pytest.approx(rhs, rel=1e-13)
    assert np.all(O.sf_back(g, ig, y)[~ig["mask"]] == 0)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("dims,deltas", [((37, 29), (1.3, 0.9)), ((64, 64), (1.0, 1.0))])
def test_footprint_size_bounds_the_sf_footprints(kind, dims, deltas):
    """footprint_size (footprint.jl:19-36) is the maximum footprint in detector samples of the
    pixels inside the radial FOV rfov = max(fovs)/2 it is computed from: their corner projections
    (tau.jl) span at most that many bins, and the widest comes within 10% of it.  (Corner pixels of a
    square image lie beyond rfov, nearer the source, and can exceed it.)"""
    g = geom(kind, nb=200, source_offset=0.0)
    ig = dict(dims=dims, deltas=deltas, offsets=(0.0, 0.0))
    (nx, ny), (dx, dy) = dims, deltas
    X, Y = np.meshgrid(dx * (np.arange(nx + 1) - nx / 2), dy * (np.arange(ny + 1) - ny / 2))
    T = O.tau(g, X.ravel(), Y.ravel()).reshape(g["na"], ny + 1, nx + 1)
    corners = np.stack([T[:, :-1, :-1], T[:, 1:, :-1], T[:, :-1, 1:], T[:, 1:, 1:]])
    width = corners.max(axis=0) - corners.min(axis=0)
    cx, cy = dx * (np.arange(nx) - (nx - 1) / 2), dy * (np.arange(ny) - (ny - 1) / 2)
    inside = np.hypot(cx[None, :], cy[:, None]) + 0.5 * math.hypot(dx, dy) <= max(nx * dx, ny * dy) / 2
    fs = O.footprint_size(g, ig)
    w = width[:, inside].max()
    assert 0.9 * fs < w <= fs * (1 + 1e-6)


def _disk_image(ig, cx, cy, r, sub=8):
    (nx, ny), (dx, dy) = ig["dims"], ig["deltas"]
    xs = dx * (np.arange(nx) - (nx - 1) / 2)
    ys = dy * (np.arange(ny) - (ny - 1) / 2)
    o = (np.arange(sub) + 0.5) / sub - 0.5
    X = (xs[None, :, None] + dx * o[None, None, :])
    Y = (ys[:, None, None] + dy * o[None, None, :])
    inside = ((X[:, :, None, :] - cx) ** 2 + (Y[:, :, :, None] - cy) ** 2) <= r * r
    return inside.mean(axis=(2, 3))


@pytest.mark.parametrize("kind", KINDS)
def test_sf_oracle_approaches_the_analytic_line_integrals(kind):
    """A finely sampled disk projected by the SF model is close to its analytic sinogram (the
    reference tests' radon(rays(rg), ob), here ellipse_sino)."""
    g = geom(kind, nb=96, d=0.9, offset=0.0, na=24, source_offset=0.0)
    ig = dict(dims=(64, 64), deltas=(1.0, 1.0), offsets=(0.0, 0.0))
    img = _disk_image(ig, 6.0, -4.0, 17.0)
    sino = O.sf_project(g, ig, img)
    ref = O.ellipse_sino(g, np.array([[6.0, -4.0, 17.0, 17.0, 0.0, 1.0]]))
    assert O.rel_rmse(sino, ref) < 0.02


def test_sf_geometry_errors_without_gpu():
    """Plan creation checks the geometry on the host before any device work."""
    ig = S.ImageGeom((64, 64), (1.0, 1.0))
    with pytest.raises(S.SinogramsError, match="0.99 dso"):
        S.SFPlan(S.SinoFanArc(nb=64, na=8, d=1.0, dsd=60.0, dod=20.0), ig)  # image corner 45 > 0.99 * 40
    with pytest.raises(ValueError):
        O.sf_project(dict(kind="arc", nb=64, d=1.0, offset=0.0, na=8, orbit=360.0, orbit_start=0.0, dsd=60.0,
                          dod=20.0, source_offset=0.0), dict(dims=(64, 64), deltas=(1.0, 1.0), offsets=(0.0, 0.0)),
                     np.ones((64, 64)))
    with pytest.raises(S.SinogramsError, match="90 degrees"):
        S.SFPlan(S.SinoFanArc(nb=700, na=8, d=1.0, dsd=200.0, dod=100.0), S.ImageGeom((8, 8), (1.0, 1.0)))  # +-100 deg
    with pytest.raises(S.SinogramsArgumentError):
        S.SFPlan(S.SinoPar(nb=64, na=8, d=-1.0), ig)
    with pytest.raises(S.SinogramsArgumentError):
        S.SFPlan(S.SinoPar(nb=64, na=8), S.ImageGeom((8, 8, 4), (1.0, 1.0, 1.0)))
    with pytest.raises(S.SinogramsArgumentError):
        S.SFPlan(S.SinoMoj(nb=64, na=8), ig)


@pytest.mark.parametrize("kind", KINDS)
def test_sf_fixture_reproduces(kind):
    """tests/golden/sf.npz (made by make_fixtures.py from the FP64 oracle) is what the oracle computes."""
    import os
    f = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sf.npz"))
    c = C.SF[kind]
    np.testing.assert_allclose(O.sf_project(c["rg"], c["ig"], f[f"{kind}_image"]), f[f"{kind}_ref_proj"], rtol=1e-12,
                               atol=1e-12)
    np.testing.assert_allclose(O.sf_back(c["rg"], c["ig"], f[f"{kind}_sino"]), f[f"{kind}_ref_back"], rtol=1e-12,
                               atol=1e-12)
