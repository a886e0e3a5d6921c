"""CPU tests of the library's host side: it loads, exports every symbol the public
header declares, and its plan-time FP64 arithmetic and error behaviour match the oracle
and the reference (no GPU needed: these entry points run on the host)."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

import cases as C
import oracle as O
import sinograms as S
from sinograms import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KA = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_known_answers.json")))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "sinogb300.h")).read()
    return sorted(set(re.findall(r"^SGB_API\s+(?:int|long long)\s+(sgb_\w+)\s*\(", txt, flags=re.M)))


def test_library_exports_every_header_symbol():
    L = _lib.lib()
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) <= set(_lib.exported_symbols())  # the ctypes table covers the header
    assert L.sgb_version() >= 10000


GEOMS = [
    S.SinoPar(), S.SinoPar(orbit=270), S.SinoPar(nb=64, d=0.5, offset=0.25, orbit=360),
    S.SinoFanArc(), S.SinoFanArc.short(), S.SinoFanFlat(nb=64, d=0.5, offset=0.25),
    S.SinoFanFlat.short(nb=96, d=0.7, dsd=300.0, dod=100.0), S.SinoFanArc.ge1(orbit="short"),
    S.CtFanArc(), S.CtFanArc.short(ns=64, nt=40, ds=1.0, dt=1.2, na=59),
    S.CtFanFlat(ns=64, nt=40, ds=1.0, dt=1.2, na=32), S.CtFanFlat.short(ns=48, nt=16, offset_s=0.25, na=40),
]


@pytest.mark.parametrize("rg", GEOMS, ids=lambda g: f"{type(g).__name__}-{g.na}")
def test_plan_time_tables_match_oracle(rg):
    for win in (S.Window(), S.Window("hann", 0.8), S.Window("hamming"), S.Window("boxcar", 0.5)):
        Hk = S.fbp_filter(rg, window=win)
        Ho = O.fbp_filter(rg, shape=win.shape, cutoff=win.cutoff)
        np.testing.assert_allclose(Hk, Ho, rtol=1e-12, atol=1e-13 * np.abs(Ho).max())
    pw, po = S.parker_weight(rg), O.parker_weight(rg)
    assert pw.shape == po.shape and np.array_equal(pw.astype(np.float64), po)
    assert S._angle_weights(S._ar(rg)) == pytest.approx(O.angle_weight(rg), rel=1e-15)
    if isinstance(rg, S.geom.CtFan):
        np.testing.assert_allclose(S.fdk_weight_cyl(rg), O.fdk_weight_cyl(rg), rtol=1e-14)
        np.testing.assert_allclose(S.fdk_view_weight(rg), O.fdk_weights(rg), rtol=1e-6)
    elif rg.kind != "par":
        np.testing.assert_allclose(S.fbp_sino_weight(rg), O.fbp_sino_weight(rg), rtol=1e-14)


def test_ramp_and_window():
    for N, ds, dsd in ((8, 2.0, 99.0), (6, 1.0, 50.0), (1024, 1.0239, 949.075)):
        np.testing.assert_allclose(S.ramp_flat(N, ds)[0], O.ramp(dict(kind="flat", ds=ds, ns=2), N), rtol=1e-15)
        np.testing.assert_allclose(S.ramp_arc(N, ds, dsd)[0], O.ramp(dict(kind="arc", ds=ds, ns=2, dsd=dsd), N),
                                   rtol=1e-14)
        assert list(S.ramp_flat(N, ds)[1]) == list(range(-(N // 2), N // 2))
    w = S.fbp_window(S.Window("hamming"), 4)
    assert np.array_equal(w.astype(np.float32), np.array(KA["window"]["hamming_N4"]["value"], np.float32))
    assert S.fbp_window(S.Window(np.arange(1, 9)), 8)[0] == 5
    for sh in ("none", "boxcar", "hamming", "hann"):
        assert S.fbp_window(S.Window(sh, 0.7), 8)[0] == 1


def test_errors_like_reference():
    with pytest.raises(S.SinogramsArgumentError, match="N must be even"):
        S.ramp_flat(7, 1.0)  # ramp.jl:87
    with pytest.raises(S.SinogramsArgumentError, match="physically impossible"):
        S.ramp_arc(4096, 1.0, 100.0)  # ramp.jl:70-72
    with pytest.raises(S.SinogramsArgumentError, match="N mismatch"):
        S.fbp_window(S.Window(np.ones(7)), 8)  # window.jl:72
    with pytest.raises(S.SinogramsArgumentError, match="Parker"):
        S.parker_weight(S.SinoPar(orbit=361))  # parker.jl:45
    with pytest.raises(S.SinogramsArgumentError, match="Unequal"):
        S._angle_weights([0.0, 0.1, 0.3])  # d-angle.jl:57


def test_geometry_defaults_match_doctests():
    d = KA["defaults"]
    for cls, key in ((S.SinoPar, "SinoPar"), (S.SinoFanArc, "SinoFanArc"), (S.CtFanArc, "CtFanArc")):
        g = cls()
        for k, v in d[key].items():
            if k != "source":
                assert getattr(g, k) == pytest.approx(v), (key, k)
    for cls, key in ((S.SinoFanArc.ge1, "SinoFanArc_ge1"), (S.CtFanArc.ge1, "CtFanArc_ge1")):
        g = cls()
        for k, v in d[key].items():
            if k != "source":
                assert getattr(g, k) == pytest.approx(v, rel=1e-6), (key, k)
    assert S.SinoFanArc.short().na == 70
    assert S.dims(S.CtFanFlat()) == (128, 64, 64)


def test_plan_validation_without_gpu():
    """Bad sizes are rejected on the host before any device work."""
    with pytest.raises(S.SinogramsArgumentError):
        S.fbp_sino_filter(np.ones((3, 40), np.float32), np.ones(32), extra=0)  # nb > npad, filter.jl:131


def test_cases_match_reference_short_constructor():
    g = C.short(dict(kind="arc", nb=128, d=1.0, offset=0.0, dsd=512.0), 128)
    assert g["na"] == S.SinoFanArc.short().na
    assert g["orbit"] == pytest.approx(S.SinoFanArc.short().orbit)


@pytest.mark.parametrize("pitch,na,orbit", [(0.5, 24, 360.0), (1.25, 37, 270.0), (0.0, 10, 360.0), (0.7, 1, 360.0)])
def test_source_zs_helix(pitch, na, orbit):
    """_source_zs / _source_dz_per_view (ct-geom.jl:118-140) from the library's host code,
    the Python mirror and the oracle restatement."""
    g = C.ct("arc", src="helix", pitch=pitch, source_z0=-3.0, na=na, orbit=orbit)
    rg = C.to_geom(g)
    zs = S._source_zs(rg)
    ref = O.source_zs(g)
    np.testing.assert_allclose(zs, ref, rtol=0, atol=1e-12)
    zfov = (g["dsd"] - g["dod"]) / g["dsd"] * g["nt"] * g["dt"]
    dz = 0.0 if na == 1 else float(np.float32(pitch)) * zfov / (na * 360 / orbit)
    assert S._source_dz_per_view(rg) == pytest.approx(dz, abs=1e-15)
    np.testing.assert_allclose(zs, np.arange(na) * dz - 3.0, rtol=0, atol=1e-12)
    assert np.all(S._source_zs(C.to_geom(C.ct("flat", na=na))) == 0)


def test_oracle_helix_shift_sign():
    """A constant source z c equals a circular scan of the grid shifted by -c in z:
    t' = mag * (z - c) (the commented cbct-back.jl:188)."""
    rg, ig = C.ct("flat", na=12), dict(dims=(8, 7, 6), deltas=(1.0, 1.0, 0.8), offsets=(0.0, 0.0, 0.25))
    proj = O.ellipsoid_proj(rg, C.ELL3)
    c = 0.6
    shifted = O.cbct_back(proj, rg, ig, zs=np.full(12, c))
    ig2 = dict(ig, offsets=(0.0, 0.0, 0.25 + c / 0.8))
    np.testing.assert_allclose(shifted, O.cbct_back(proj, rg, ig2), rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(O.cbct_back(proj, rg, ig, zs=None), O.cbct_back(proj, rg, ig))


def test_zwart_powell_known_answers():
    """test/sys2/zwart_powell.jl:11-13 -- zwart_powell(0, 0) == 0.75, zwart_powell(0, pi/4)
    ~ 1/sqrt(2) -- from the library and the oracle, and library == oracle on the test grid."""
    assert S.zwart_powell(0, 0) == 0.75
    assert S.zwart_powell(0, np.pi / 4) == pytest.approx(1 / np.sqrt(2), rel=1e-12)
    assert O.zwart_powell(0, 0) == pytest.approx(0.75, rel=1e-14)
    r = np.linspace(-1, 1, 101) * 2
    phi = np.linspace(0, np.pi, 181)
    R, P = np.meshgrid(r, phi)
    np.testing.assert_allclose(S.zwart_powell(R, P), O.zwart_powell(R, P), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("case", [
    dict(g=dict(kind="par", nb=64, d=0.7, offset=0.25, na=10, orbit=180.0), ig=dict(dims=(40, 30), deltas=(0.5, 0.6))),
    dict(g=dict(kind="arc", nb=888, d=1.0239, offset=1.25, na=10, orbit=360.0, dsd=949.075, dod=408.075,
                source_offset=0.0), ig=dict(dims=(512, 512), deltas=(0.9766, 0.9766))),
    dict(g=dict(kind="flat", nb=910, d=1.0239, offset=0.0, na=10, orbit=360.0, dsd=949.0, dod=408.0,
                source_offset=0.0), ig=dict(dims=(256, 200), deltas=(2.0, 2.0))),
    dict(g=C.ct("flat", offset_s=0.25), ig=dict(dims=(16, 14, 12), deltas=(1.0, 1.1, 0.9))),
    dict(g=C.ct("arc"), ig=dict(dims=(20, 20, 8), deltas=(2.0, 2.0, 1.0))),
])
def test_footprint_size(case):
    """footprint_size (footprint.jl:19-36) from the library against the oracle restatement."""
    g, ig = case["g"], case["ig"]
    got = S.footprint_size(C.to_geom(g), C.to_image(ig))
    assert got == O.footprint_size(g, ig)
    assert got > 0


def test_footprint_size_bad_dso():
    """rfov > 0.99 dso throws "bad dso" (footprint.jl:28, :34)."""
    g = C.ct("flat", dsd=40.0, dod=10.0)  # dso 30 < rfov 40
    with pytest.raises(S.SinogramsError, match="bad dso"):
        S.footprint_size(C.to_geom(g), C.to_image(dict(dims=(80, 80, 4), deltas=(1.0, 1.0, 1.0))))
    with pytest.raises(ValueError, match="bad dso"):
        O.footprint_size(g, dict(dims=(80, 80, 4), deltas=(1.0, 1.0, 1.0)))


@pytest.mark.parametrize("detector", ["arc", "flat"])
def test_learned_ramp_gain_file_and_round_trip(tmp_path, detector):
    """The committed learned-ramp gain is even (a real, symmetric row filter), passes DC and
    only attenuates; a saved gain loads back unchanged; a gain of the wrong length is refused."""
    from sinograms import learned as LF
    lr = LF.LearnedRamp.load(LF.default_ramp_path(detector))
    g = lr.gain
    assert g.shape == (lr.npad,) and np.array_equal(g[1:], g[1:][::-1])
    assert abs(g[0] - 1.0) < 1e-3 and g.max() < 1.01 and g.min() > 0.0
    p = str(tmp_path / "g.npz")
    lr.save(p)
    back = LF.LearnedRamp.load(p)
    assert np.array_equal(back.gain, g) and back.npad == lr.npad and back.meta["phantoms"] == lr.meta["phantoms"]
    with pytest.raises(S.SinogramsArgumentError):
        LF.LearnedRamp(g[:-1], lr.npad)


def test_learned_training_schedule_resumes_where_it_stopped():
    """train(start=k) after train(stop=k) takes the same batches at the same rates as one
    uninterrupted run (the seeded shuffles of finished epochs are drawn again), so a filter
    restored from a checkpoint continues the schedule it was saved in."""
    import torch
    from sinograms import learned as LF

    class Recorder:  # stands in for the GPU filter: records each step's rows and rate
        def __init__(self):
            self.steps = []

        def train_step(self, z, t, rate):
            self.steps.append((z[:, 0].tolist(), rate))
            return 0.0

    zn = torch.arange(1000, dtype=torch.float32)[:, None].repeat(1, 3)
    full = Recorder()
    LF.train(full, zn, zn, epochs=3, batch=64, seed=7)
    assert len(full.steps) == 3 * (1000 // 64)
    for k in (1, 15, 16, 31, 44):
        a, b = Recorder(), Recorder()
        LF.train(a, zn, zn, epochs=3, batch=64, seed=7, stop=k)
        LF.train(b, zn, zn, epochs=3, batch=64, seed=7, start=k)
        assert a.steps + b.steps == full.steps, k


def test_learned_filter_refuses_params_of_the_wrong_size():
    """sgb_lf_create reads nparam floats from its pointer, so the host side checks the count
    (the network's shape gives it; the FP64 oracle of the network agrees) before the call."""
    import learned_oracle as LO
    from sinograms import learned as LF
    assert LF.NPARAM == LO.nparams() == 28353
    with pytest.raises(ValueError):
        LF.LearnedFilter(scale=1.0, params=np.zeros(LF.NPARAM - 1, np.float32))


def test_output_buffers_are_checked_before_the_library_writes():
    """A caller's `out` must hold exactly the prod(shape) float32 values the library writes, on
    the input's side; anything else raises instead of letting the call write out of bounds."""
    import torch
    from sinograms._arrays import Arr, check_out, out_buffer
    host = Arr(np.zeros((4, 6), np.float32))
    good = np.empty((3, 5), np.float32)
    assert out_buffer(good, (3, 5), host) is good
    assert out_buffer(None, (3, 5), host).shape == (3, 5)
    t = torch.empty((3, 5))
    assert check_out(t, (3, 5), device=False) is t
    for bad in (np.empty((3, 4), np.float32), np.empty((3, 5), np.float64), np.empty((5, 3), np.float32).T,
                torch.empty((3, 5), dtype=torch.float64), [0.0] * 15):
        with pytest.raises(ValueError):
            out_buffer(bad, (3, 5), host)
    with pytest.raises(ValueError):  # a host array cannot take a device call's output
        check_out(good, (3, 5), device=True)


def test_cbct_back_refuses_projections_that_do_not_match_the_geometry():
    """cbct_back takes one view angle per projection from rg, so a proj whose size differs from
    dims(rg) is refused before the library is called (cbct-back.jl:116 checks the image sizes)."""
    rg = S.CtFanFlat(ns=40, nt=30, na=25, ds=1.0, dt=1.0, dsd=500.0, dod=200.0)
    ig = S.ImageGeom((20, 18, 14), (1.0, 1.0, 1.0))
    with pytest.raises(S.SinogramsArgumentError):
        S.cbct_back(np.zeros((26, 30, 40), np.float32), rg, ig)
    with pytest.raises(S.SinogramsArgumentError):
        S.cbct_back(np.zeros((25, 30, 40), np.float32), rg, S.ImageGeom((20, 18), (1.0, 1.0)))


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_public_header_compiles_alone(tmp_path, lang):
    """include/sinogb300.h is plain C (no CUDA or torch types): it compiles on its own as C99
    and as C++17, as a host program binding the library would include it."""
    import shutil
    import subprocess
    cc = "gcc" if lang == "c" else "g++"
    if shutil.which(cc) is None:
        pytest.skip(f"{cc} not found")
    src = tmp_path / "use_header.c"
    src.write_text('#include "sinogb300.h"\nint main(void) { return sgb_version() > 0 ? 0 : 1; }\n')
    std = "-std=c99" if lang == "c" else "-std=c++17"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([cc, std, "-x", lang, "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                        "-I", os.path.join(root, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_sinomoj_geometry_ramp_and_parker():
    """SinoMoj (type2.jl:112-121): the doctest defaults (type2.jl:205-213), fbp_ramp with its
    `dr` keyword (ramp.jl:27-30; test/fbp/ramp.jl:40-52 asks for N samples for every 2D type),
    the Parker weight (parker.jl:122-129) and the per-view ray spacing (common.jl:128-129).
    The reference has no FBP plan for it, and neither has this library."""
    g = S.SinoMoj()
    assert (g.nb, g.d, g.offset, g.na, g.orbit, g.orbit_start) == (128, 1.0, 0.0, 200, 180.0, 0.0)
    assert S.dims(g) == (128, 200)
    rg = S.SinoMoj(d=2.0, orbit=90.0)
    h, n = S.fbp_ramp(rg, 8)
    assert len(h) == 8 and len(n) == 8
    np.testing.assert_array_equal(h, S.ramp_flat(8, 2.0)[0])
    np.testing.assert_array_equal(S.fbp_ramp(rg, 8, dr=0.5)[0], S.ramp_flat(8, 0.5)[0])
    with pytest.raises(S.SinogramsArgumentError):
        S.fbp_ramp(S.SinoPar(), 8, dr=0.5)
    np.testing.assert_array_equal(S.fbp_filter(S.SinoMoj(nb=100, d=0.7)), S.fbp_filter(S.SinoPar(nb=100, d=0.7)))
    assert S.parker_weight(S.SinoMoj(orbit=360.0)).shape == (1, 1)
    with pytest.raises(S.SinogramsArgumentError):
        S.parker_weight(S.SinoMoj(orbit=270.0))
    d = S._d_ang(S.SinoMoj(d=2.0, na=4, orbit=180.0))  # views at 0, 45, 90, 135 degrees
    np.testing.assert_allclose(d, [2.0, 2.0 / np.sqrt(2), 2.0, 2.0 / np.sqrt(2)], rtol=1e-12)
    with pytest.raises(NotImplementedError):
        S.plan_fbp(g, S.ImageGeom((64, 64), (1.0, 1.0)))


def test_learned_state_entry_points_check_arguments_without_a_gpu():
    """sgb_lf_get_state / sgb_lf_set_state refuse a missing handle or buffer and a negative
    step with SGB_ERR_ARG and a message, before any device work."""
    L = _lib.lib()
    buf = np.zeros(4, np.float32)
    p = buf.ctypes.data_as(ctypes.c_void_p)
    assert L.sgb_lf_get_state(None, p, p, None) == _lib.SGB_ERR_ARG
    assert "lf_get_state" in _lib.last_error()
    assert L.sgb_lf_set_state(None, p, p, 3) == _lib.SGB_ERR_ARG
    assert "lf_set_state" in _lib.last_error()
