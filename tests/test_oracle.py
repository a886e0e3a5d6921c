"""Pins the CPU oracle to the reference's own known answers and conservation tests
(tests/golden/reference_known_answers.json, read from the Sinograms.jl test suite) and
checks that the committed golden fixtures still reproduce."""
import json
import math
import os

import numpy as np
import pytest

import cases as C
import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "reference_known_answers.json")))


def sino(**kw):
    g = dict(kind="par", nb=128, d=1.0, offset=0.0, na=200, orbit=180.0, orbit_start=0.0, source_offset=0.0,
             dsd=512.0, dod=128.0)
    g.update(kw)
    return g


def test_window_known_answers():
    w = O.window(4, "hamming")
    assert np.array_equal(w.astype(np.float32), np.array(KA["window"]["hamming_N4"]["value"], np.float32))
    for sh in KA["window"]["first_sample_cutoff_0p7_N8"]["shapes"]:
        assert O.window(8, sh, 0.7)[0] == 1.0
    assert O.window(8, "vect", vect=np.arange(1, 9))[0] == KA["window"]["windowvect_1to8_first"]["value"]


def _ar32(g):
    """The reference's Float32 angles: range(orbit_start, length=na, step=orbit/na) in
    Float32, times Float32(deg2rad(1)) (common.jl:27-34, unit.jl:10)."""
    deg = (np.float64(g["orbit_start"]) + np.arange(g["na"]) * (np.float64(np.float32(g["orbit"])) / g["na"]))
    return (deg.astype(np.float32) * np.float32(math.pi / 180)).astype(np.float32)


def _aw(ar):
    import ctypes
    a = np.ascontiguousarray(ar, dtype=np.float64)
    w = ctypes.c_double()
    rtol = ctypes.c_double(float(np.sqrt(np.finfo(np.float32).eps)))  # isapprox on Float32 angles
    assert O.lib().orc_angle_weight_tol(ctypes.c_void_p(a.ctypes.data), len(a), rtol, ctypes.byref(w)) == 0
    return w.value


def test_angle_weight_known_answers():
    """The doctest values are Float32 results: the oracle's formula applied to the
    reference's Float32 angles reproduces them exactly."""
    a = KA["angle_weights"]
    assert np.float32(_aw(_ar32(sino()))) == np.float32(a["SinoPar_default"]["value"])
    assert np.float32(_aw(_ar32(sino(orbit=360.0)))) == np.float32(a["SinoPar_orbit360"]["value"])
    g = C.short(sino(kind="arc", orbit=360.0), 128)
    assert g["na"] == 70
    g = dict(g, orbit=float(np.float32(g["orbit"])))
    assert np.float32(_aw(_ar32(g))) == pytest.approx(np.float32(a["SinoFanArc_short"]["value"]), rel=1.2e-7)
    assert O.angle_weight(sino()) == pytest.approx(a["SinoPar_default"]["value"], rel=2e-7)
    g = sino(orbit=-720.0, orbit_start=100.0)
    assert O.angle_weight(g) == pytest.approx(math.pi / g["na"], rel=3.5e-4)
    ge = sino(kind="arc", nb=888, d=1.0239, offset=1.25, na=642, orbit=642 / 984 * 360, dsd=949.075, dod=408.075)
    assert O.angle_weight(ge) == pytest.approx(math.pi / ge["na"] * ge["orbit"] / 180, rel=3.5e-4)


def test_parker_known_answers():
    p = KA["parker"]
    pw = O.parker_weight(sino(orbit=270.0))
    assert pw.shape[::-1] == tuple(p["SinoPar_orbit270"]["size"])
    assert pw.ravel()[0] == p["SinoPar_orbit270"]["first"]
    assert pw.mean() == pytest.approx(p["SinoPar_orbit270"]["mean_approx"], rel=p["SinoPar_orbit270"]["rtol"])
    ge = sino(kind="arc", nb=888, d=1.0239, offset=1.25, na=642, orbit=float(np.float32(642 / 984 * 360)),
              dsd=949.075, dod=408.075)
    rs = O.parker_weight(ge).astype(np.float32).sum(axis=0)
    assert 1 - rs.min() / rs.max() < p["SinoFanArc_ge1_short_rowsum_spread_lt"]["value"]
    assert O.parker_weight(sino(kind="arc", orbit=360.0)).shape == (1, 1)
    ct = C.ct("arc", ns=128, nt=64, na=64, dsd=512.0, dod=128.0, dt=1.0)
    assert O.parker_weight(ct).shape == tuple(p["CtFanArc_default_size"]["value"])
    assert O.parker_weight(C.short(ct, 128)).shape[1] == p["CtFanArc_short_dim2"]["value"]


def test_filter_length():
    assert len(O.fbp_filter(sino())) == KA["filter"]["SinoPar_nb128_length"]["value"]


def test_sino_filter_equals_fft():
    """The oracle's direct circular convolution equals the reference's padded-FFT
    product (filter.jl:133-144), with and without wrap-around."""
    rng = np.random.default_rng(0)
    for nb, npad in ((24, 32), (40, 128), (33, 64)):
        x = rng.standard_normal((7, nb))
        Hk = O.fbp_filter(sino(nb=nb), npad=npad, shape="hann")
        pad = np.zeros((7, npad))
        pad[:, :nb] = x
        ref = np.real(np.fft.ifft(np.fft.fft(pad, axis=1) * Hk, axis=1))[:, :nb]
        assert np.allclose(O.sino_filter(x, Hk), ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def _disk_area_err(rec, dx):
    return abs(rec.sum() * dx * dx - math.pi * 4) / (math.pi * 4)


def test_fbp_par_conservation():
    c = KA["conservation"]["fbp_par_convenience"]
    nr, dr = c["nr"], c["fov"] / c["nr"]
    g = sino(nb=nr, d=dr, na=c["na"])
    s = O.ellipse_sino(g, np.array([[2.0, 1.0, 2.0, 2.0, 0.0, 1.0]])).astype(np.float32)
    ax = O.image_axes(dict(dims=(nr, nr), deltas=(dr, dr)))
    mask = (ax[0][None, :] ** 2 + ax[1][:, None] ** 2) <= O.rfov(g) ** 2
    rec = O.fbp(g, dict(dims=(nr, nr), deltas=(dr, dr), mask=mask), s)
    assert _disk_area_err(rec, dr) < c["area_err_lt"]
    c = KA["conservation"]["fbp_par_plan"]
    g = sino(d=c["d"])
    s = O.ellipse_sino(g, np.array([[2.0, 1.0, 2.0, 2.0, 0.0, 1.0]])).astype(np.float32)
    ax = O.image_axes(dict(dims=(128, 128), deltas=(0.1, 0.1)))
    ig = dict(dims=(128, 128), deltas=(0.1, 0.1), mask=(ax[0][None, :] ** 2 + ax[1][:, None] ** 2) <= O.rfov(g) ** 2)
    for k in c["linearity"]:
        assert _disk_area_err(O.fbp(g, ig, k * s) / k, 0.1) < c["area_err_lt"]


@pytest.mark.parametrize("kind", ["arc", "flat"])
@pytest.mark.parametrize("short", [False, True])
def test_fbp_fan_conservation(kind, short):
    c = KA["conservation"]["fbp_fan"]
    g = sino(kind=kind, d=c["d"], orbit=360.0, dsd=51.2, dod=12.8)
    if short:
        g = C.short(g, 128)
    ax = O.image_axes(dict(dims=(128, 128), deltas=(0.1, 0.1)))
    ig = dict(dims=(128, 128), deltas=(0.1, 0.1), mask=(ax[0][None, :] ** 2 + ax[1][:, None] ** 2) <= O.rfov(g) ** 2)
    s = O.ellipse_sino(g, np.array([[2.0, 1.0, 2.0, 2.0, 0.0, 1.0]])).astype(np.float32)
    assert _disk_area_err(O.fbp(g, ig, s), 0.1) < c["area_err_lt"]


@pytest.mark.parametrize("kind", ["arc", "flat"])
@pytest.mark.parametrize("short", [False, True])
def test_fdk_conservation(kind, short):
    c = KA["conservation"]["fdk"]
    rg = C.ct(kind, ns=c["ns"], nt=c["nt"], ds=c["ds"], dt=c["dt"], na=c["na_full"], dsd=4 * 64.0, dod=64.0)
    if short:
        rg = C.short(rg, c["na_short"])
    e = c["ellipsoid"]
    proj = O.ellipsoid_proj(rg, np.array([e + [0.0, 0.0, 0.0, 1.0]])).astype(np.float32)
    rec = O.fdk(rg, dict(dims=tuple(c["ig"]), deltas=(1.0, 1.0, 1.0)), proj)
    vt = 4 / 3 * math.pi * e[3] * e[4] * e[5]
    assert abs(rec.sum() - vt) / vt < (c["vol_err_lt_short"] if short else c["vol_err_lt_full"])


def test_bdd_adjoint():
    c = KA["conservation"]["bdd_adjoint"]
    down = c["down"]
    nb, d, na = 2 * max(c["nb"] // (2 * down), 1), c["d"] * down, c["na"] // down
    geo = O.bdd_geo(c["dsd"], c["dsd"] - c["dod"], c["dx"] * down, d, c["npix"] // down, nb,
                    np.arange(na) * (2 * math.pi / na))
    rng = np.random.default_rng(0)
    x, y = rng.random((geo["nPix"],) * 2), rng.random((nb, na))
    lhs = np.dot(O.project_bdd(x, geo).ravel(), y.ravel())
    rhs = np.dot(x.ravel(), O.backproject_bdd(y, geo).ravel())
    assert lhs == pytest.approx(rhs, rel=c["rtol"])


def test_fixtures_reproduce():
    f = np.load(os.path.join(HERE, "golden", "fdk_flat.npz"))
    c = C.FDK_FLAT
    assert np.allclose(O.fdk(c["rg"], c["ig"], f["proj"]), f["ref"], rtol=1e-12, atol=1e-12)
    f = np.load(os.path.join(HERE, "golden", "bdd.npz"))
    g = C.BDD
    geo = O.bdd_geo(g["DSD"], g["DS0"], g["pSize"], g["dSize"], g["nPix"], g["nDet"], g["angle"])
    assert np.allclose(O.project_bdd(f["phantom"], geo), f["ref_proj"], rtol=1e-12)
    assert np.allclose(O.backproject_bdd(f["sino"], geo), f["ref_back"], rtol=1e-12)


def test_oracle_fp32_build_close_to_fp64():
    c = C.FDK_FLAT
    f = np.load(os.path.join(HERE, "golden", "fdk_flat.npz"))
    r32 = O.fdk(c["rg"], c["ig"], f["proj"], bits=32)
    assert O.rel_rmse(r32, f["ref"]) < 1e-5


def test_learned_oracle_gradient_finite_differences():
    """The FP64 network restatement's analytic gradient matches central differences."""
    import learned_oracle as LO
    rng = np.random.default_rng(11)
    p = 0.3 * rng.standard_normal(LO.nparams())
    z, t = rng.standard_normal((3, 20)), rng.standard_normal((3, 20))
    loss, g = LO.loss_grad(p, z, t, 0.7, bf16_weights=False)
    for i in rng.choice(p.size, 25, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-5
        fd = (LO.loss_grad(p + e, z, t, 0.7, False)[0] - LO.loss_grad(p - e, z, t, 0.7, False)[0]) / 2e-5
        assert fd == pytest.approx(g[i], rel=1e-6, abs=1e-9 * np.abs(g).max())
