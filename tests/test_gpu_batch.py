"""Batched FDK (one CUDA graph, one persistent back-projection launch over many scans):
every scan must equal its own single-scan plan and the FP64 oracle."""
import numpy as np
import pytest

import cases as C
import oracle as O
import sinograms as S

pytestmark = pytest.mark.gpu


def _scans():
    rgs = [S.CtFanFlat(ns=61, nt=40, ds=1.0, dt=1.1, na=37, dsd=220.0, dod=70.0, offset_s=0.25),
           S.CtFanArc(ns=48, nt=32, ds=1.2, dt=1.0, na=24, dsd=180.0, dod=60.0),
           S.CtFanArc.short(ns=40, nt=24, ds=1.0, dt=1.0, na=30, dsd=150.0, dod=50.0),
           S.CtFanFlat(ns=80, nt=20, ds=0.9, dt=1.3, na=50, dsd=300.0, dod=100.0, offset_t=-0.5),
           S.CtFanFlat(ns=33, nt=30, ds=1.0, dt=1.0, na=19, dsd=140.0, dod=40.0)]
    igs = [S.ImageGeom((21, 19, 13), (1.0, 1.0, 1.1), (0.3, 0.0, 0.0)),
           S.ImageGeom((32, 32, 16), (1.1, 1.1, 1.0)),
           S.ImageGeom((18, 18, 9), (1.0, 1.0, 1.0)),
           S.ImageGeom((40, 24, 11), (1.0, 1.0, 1.0)),
           S.ImageGeom((16, 17, 20), (0.9, 0.9, 0.8))]
    ig3 = igs[3]
    igs[3] = ig3.with_mask(ig3.circle(10.0))
    return rgs, igs


def _oracle_geom(rg):
    return dict(kind=rg.kind, ns=rg.ns, nt=rg.nt, ds=rg.ds, dt=rg.dt, offset_s=rg.offset_s, offset_t=rg.offset_t,
                na=rg.na, orbit=rg.orbit, orbit_start=rg.orbit_start, source_offset=0.0, dsd=rg.dsd, dod=rg.dod)


@pytest.mark.parametrize("storage", ["f32", "bf16", "f16"])
def test_batch_equals_single_scan_plans(cuda, storage):
    rgs, igs = _scans()
    batch = S.FDKBatch(rgs, igs, storage=storage)
    info = batch.info()
    assert info["scans"] == len(rgs) and info["ctas"] > 0
    assert len(info["classes"]) == info["launches"] and info["classes"][0]["ctas"] == info["ctas"]
    for c in info["classes"]:
        assert c["box_width"] in (32, 64, 128) and c["zu"] in (16, 32, 64) and c["views_per_stage"] in (1, 2, 4)
        assert c["sample_bytes"] in (2, 4, 8) and c["ctas"] > 0 and c["mupdates"] >= 0 and c["stages"] in (2, 4)
    assert abs(sum(c["mupdates"] for c in info["classes"]) * 1e6 - info["updates"]) <= 0.5e6 * len(info["classes"])
    projs = [S.ellipsoid_proj(rg, C.ELL3) for rg in rgs]
    for i, p in enumerate(projs):
        batch.set_input(i, p)
    for rep in range(2):  # the graph replays
        batch.run()
        for i, (rg, ig, p) in enumerate(zip(rgs, igs, projs)):
            out = batch.get_output(i)
            single = S.fdk(S.plan_fbp(rg, ig, storage=storage), p)
            err = O.rel_rmse(out, single)
            # FP32 and BF16: the same arithmetic whatever the z-unroll.  F16 quads: the t-weights are
            # rounded to a 2^-10 grid from the z-tile's first voxel, so a batch and a plan with
            # different z-unrolls round them independently; they agree within half the form's own
            # error bar against FP64 (test_batch_against_oracle holds each to the full bar)
            bar = 0.5 * C.form_bars("f16", rg.na)[0] if storage == "f16" else 1e-5
            assert err < bar, (i, rep, err)
            if ig.mask is not None:
                assert np.all(out[~ig.mask] == 0)


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_batch_against_oracle(cuda, storage):
    rgs, igs = _scans()
    batch = S.FDKBatch(rgs, igs, storage=storage)
    projs = [S.ellipsoid_proj(rg, C.ELL3) for rg in rgs]
    for i, p in enumerate(projs):
        batch.set_input(i, p)
    batch.run()
    for i, (rg, ig, p) in enumerate(zip(rgs, igs, projs)):
        ref = O.fdk(_oracle_geom(rg), dict(dims=ig.dims, deltas=ig.deltas, offsets=ig.offsets, mask=ig.mask), p)
        out = batch.get_output(i)
        rmse, maxrel = C.form_bars(storage, rg.na)
        assert O.rel_rmse(out, ref) < rmse, i
        assert np.abs(out - ref).max() <= maxrel * np.abs(ref).max(), i


def test_batch_rejects_too_many_scans():
    rgs = [S.CtFanFlat(ns=16, nt=8, na=8)] * 65
    igs = [S.ImageGeom((8, 8, 4))] * 65
    with pytest.raises(S.SinogramsArgumentError):
        S.FDKBatch(rgs, igs)


def test_batch_every_box_class_reruns_with_new_inputs(cuda):
    """The uneven 48-scan workload (its geometry; 24 views per scan) spreads over more than
    four persistent launches.  A second run with every input doubled must give exactly twice
    the first run's volumes in every scan (each launch's work counter is reset per run), each
    scan must match its own single-scan plan, and the FP64 oracle bounds both."""
    import torch
    rgs, igs, ells = S.random_ct_scans(48, 4)
    rgs = [type(rg)(ns=rg.ns, nt=rg.nt, ds=rg.ds, dt=rg.dt, na=24, dsd=rg.dsd, dod=rg.dod) for rg in rgs]
    batch = S.FDKBatch(rgs, igs)
    info = batch.info()
    assert info["launches"] > 4, info["classes"]
    projs = [S.ellipsoid_proj(rg, e, device=True) for rg, e in zip(rgs, ells)]
    for i, p in enumerate(projs):
        batch.set_input(i, p)
    batch.run()
    first = [batch.get_output(i) for i in range(len(rgs))]
    for i, p in enumerate(projs):
        batch.set_input(i, 2 * p)
    batch.run()
    for i in range(len(rgs)):
        assert np.array_equal(batch.get_output(i), 2 * first[i]), i
    # Batch and single-scan plans may pick different z-unrolls (the batch keeps two CTAs per SM,
    # the single plan is autotuned); the t coordinate bt = bt0 + k dbt is then rounded from a
    # different base, which moves taps by ~1e-5 row on these coarse, 24-view scans.  So the
    # volumes agree to 5e-5, and the scan that differs most is checked against the FP64 oracle
    # on a central 4-slice slab, where both must meet the FP32 bar.
    diffs = []
    for i, (rg, ig, p) in enumerate(zip(rgs, igs, projs)):
        single = S.fdk(S.plan_fbp(rg, ig), p).cpu().numpy()
        diffs.append(O.rel_rmse(first[i], single))
        assert diffs[-1] < 5e-5, (i, diffs[-1])
    i = int(np.argmax(diffs))
    rg, ig, p = rgs[i], igs[i], projs[i]
    single = S.fdk(S.plan_fbp(rg, ig), p).cpu().numpy()
    nz, m = ig.dims[2], 4
    z0 = (nz - m) // 2
    slab = dict(dims=(ig.dims[0], ig.dims[1], m), deltas=ig.deltas,
                offsets=(0.0, 0.0, (nz - 1) / 2 - (m - 1) / 2 - z0))
    ref = O.fdk(_oracle_geom(rg), slab, p.cpu().numpy())
    assert O.rel_rmse(first[i][z0:z0 + m], ref) < 1e-4, (i, diffs[i])
    assert O.rel_rmse(single[z0:z0 + m], ref) < 1e-4, (i, diffs[i])
