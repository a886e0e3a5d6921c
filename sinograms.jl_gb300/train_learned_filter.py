"""Train the learned row filter on the GPU (the library's own forward/backward/Adam
kernels) and evaluate it against plain ramp FBP on held-out scans.

    python sinograms.jl_gb300/train_learned_filter.py [--phantoms 20000] [--out PATH]
    python sinograms.jl_gb300/train_learned_filter.py --linear [--phantoms 2000] [--out PATH]

Checkpoint and resume: `--stop K --checkpoint PATH` ends after K steps of the schedule and saves
params, scale and Adam state; `--resume PATH` (with the same data arguments) continues from there.

--linear fits the learned linear filter instead (LearnedRamp: the ramp response times the
least-squares per-frequency gain) and compares it with plain FBP at the same latency.

Data: seeded random-ellipse phantoms (20 ellipses, centres r <= 220 mm, semi-axes
U[4,120] mm, density U[-0.3,1]) rasterised on the 512^2 grid, projected by the
distance-driven projector over 90 views of the sparse fan geometry (arc detector unless
--detector flat), plus Gaussian noise
(sigma = 0.5% of each sinogram's peak).  Target: the plan's ramp-filtered rows of the
noise-free sinogram.  Prints one JSON summary line.
"""
import argparse
import json
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import numpy as np  # noqa: E402
import torch  # noqa: E402

import sinograms as S  # noqa: E402
from sinograms import learned as LF  # noqa: E402


def evaluate(lf, plan, rg, ig, n, seed=900000):
    geo = S.BddGeo.from_geoms(rg, ig)
    mask = torch.as_tensor(ig.mask, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(seed)
    rows = []
    for i in range(n):
        img = LF.ellipse_image(ig.with_mask(None), LF.phantom_ellipses(seed + i))
        s = LF.dd_project(img, geo)
        s = s + 0.005 * s.abs().max() * torch.randn(s.shape, device="cuda", generator=g)
        plain = S.fbp(plan, s)
        learned = LF.fbp_backproject(plan, lf.apply(LF.fbp_filter_rows(plan, s)))
        _, info = LF.fbp_learned(plan, lf, s, judge=True)
        rows.append(dict(rmse_plain=float(((plain - img)[mask]).pow(2).mean().sqrt()),
                         rmse_learned=float(((learned - img)[mask]).pow(2).mean().sqrt()), **info))
    return rows


def latency(fn, reps=20):
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def summary(lf, plan, rg, ig, n):
    """Image RMSE against the phantom, judge decisions and reprojection residuals on n held-out
    scans, and the latency of one 90-view reconstruction: plain FBP against filter rows ->
    learned filter -> back-projection, each enqueued without a host synchronisation."""
    ev = evaluate(lf, plan, rg, ig, n)
    s = LF.dd_project(LF.ellipse_image(ig.with_mask(None), LF.phantom_ellipses(1)), S.BddGeo.from_geoms(rg, ig))
    lat_plain = latency(lambda: S.fbp(plan, s, sync=False))
    lat_learned = latency(lambda: LF.fbp_backproject(
        plan, lf.apply(LF.fbp_filter_rows(plan, s, sync=False), sync=False), sync=False))
    return {
        "rmse_plain": float(np.mean([r["rmse_plain"] for r in ev])),
        "rmse_learned": float(np.mean([r["rmse_learned"] for r in ev])),
        "judge_kept_learned": int(sum(r["used"] == "learned" for r in ev)), "eval_scans": len(ev),
        "residual_plain": float(np.mean([r["residual_plain"] for r in ev])),
        "residual_learned": float(np.mean([r["residual_learned"] for r in ev])),
        "latency_ms_plain": lat_plain, "latency_ms_learned": lat_learned}


def linear_summary(lr, rg, ig, n, seed=900000):
    """Held-out image RMSE, judge decisions and latency of the learned-ramp plan against the
    plain plan (both one fbp call enqueued without a host synchronisation)."""
    plain = S.plan_fbp(rg, ig)
    learned = lr.plan(rg, ig)
    geo = S.BddGeo.from_geoms(rg, ig)
    mask = torch.as_tensor(ig.mask, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(seed)
    rp, rl, kept = [], [], 0
    for i in range(n):
        img = LF.ellipse_image(ig.with_mask(None), LF.phantom_ellipses(seed + i))
        s = LF.dd_project(img, geo)
        s = s + 0.005 * s.abs().max() * torch.randn(s.shape, device="cuda", generator=g)
        rp.append(float(((S.fbp(plain, s) - img)[mask]).pow(2).mean().sqrt()))
        rl.append(float(((S.fbp(learned, s) - img)[mask]).pow(2).mean().sqrt()))
        kept += LF.fbp_learned_ramp(learned, plain, s)[1]["used"] == "learned"
    return {"rmse_plain": float(np.mean(rp)), "rmse_learned_ramp": float(np.mean(rl)),
            "judge_kept_learned": int(kept), "eval_scans": n,
            "latency_ms_plain": latency(lambda: S.fbp(plain, s, sync=False)),
            "latency_ms_learned_ramp": latency(lambda: S.fbp(learned, s, sync=False))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--phantoms", type=int, default=20000)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--epochs", type=int, default=2)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval", type=int, default=32)
    ap.add_argument("--out", default=LF.default_weights_path())
    ap.add_argument("--eval-only", action="store_true", help="evaluate the weights at --out without training")
    ap.add_argument("--linear", action="store_true", help="fit the learned linear (ramp) filter instead")
    ap.add_argument("--checkpoint", help="save params, scale and Adam state here when the run stops")
    ap.add_argument("--stop", type=int, help="stop after this many steps of the schedule (with --checkpoint)")
    ap.add_argument("--resume", help="continue the schedule from a checkpoint (same data arguments)")
    ap.add_argument("--detector", default="arc", choices=["arc", "flat"],
                    help="SinoFanArc (the workload's geometry) or SinoFanFlat")
    args = ap.parse_args()
    rg, ig = LF.sparse_fan_geometry(detector=args.detector)
    if args.out == LF.default_weights_path():
        args.out = LF.default_weights_path(args.detector)
    if args.linear:
        out = args.out if args.out != LF.default_weights_path(args.detector) else LF.default_ramp_path(args.detector)
        if args.eval_only:
            lr = LF.LearnedRamp.load(out)
        else:
            t0 = time.perf_counter()
            lr = LF.fit_learned_ramp(args.phantoms, args.seed, rg, ig)
            lr.meta["fit_seconds"] = time.perf_counter() - t0
            os.makedirs(os.path.dirname(out), exist_ok=True)
            lr.save(out)
        print(json.dumps({"weights": out, **lr.meta, **linear_summary(lr, rg, ig, args.eval)}))
        return
    plan = S.plan_fbp(rg, ig)
    if args.eval_only:
        lf = LF.LearnedFilter.load(args.out)
        print(json.dumps({"weights": args.out, **summary(lf, plan, rg, ig, args.eval)}))
        return
    t0 = time.perf_counter()
    zn, zc = LF.make_dataset(args.phantoms, args.seed, rg, ig)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    scale = float(zc.pow(2).mean().sqrt())
    if args.resume:
        lf = LF.LearnedFilter.load_checkpoint(args.resume)
        start = lf.adam_state()[2]
    else:
        lf = LF.LearnedFilter(scale=scale, seed=args.seed)
        start = 0
    steps = args.epochs * (zn.shape[0] // args.batch)
    t0 = time.perf_counter()
    losses = LF.train(lf, zn, zc, epochs=args.epochs, batch=args.batch, lr=args.lr, seed=args.seed, start=start,
                      stop=args.stop)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del zn, zc
    if args.checkpoint:
        lf.save_checkpoint(args.checkpoint)
    done = lf.adam_state()[2]
    if done < steps:  # a partial run leaves the weights file alone
        print(json.dumps({"steps_done": done, "steps_total": steps, "checkpoint": args.checkpoint,
                          "loss_last": float(np.mean(losses[-20:])) if losses else None}))
        return
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    lf.save(args.out)
    print(json.dumps({
        "phantoms": args.phantoms, "rows": args.phantoms * rg.na, "epochs": args.epochs, "batch": args.batch,
        "steps": len(losses), "data_seconds": t_data, "train_seconds": t_train, "scale": lf.scale,
        "loss_first": losses[0], "loss_last": float(np.mean(losses[-20:])), "weights": args.out,
        **summary(lf, plan, rg, ig, args.eval)}))


if __name__ == "__main__":
    main()
