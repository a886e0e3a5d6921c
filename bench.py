"""Benchmark: FDK voxel-view updates/s on one GB300: plain FP32 form against the reduced-precision
storage forms (F16 quads, the headline at <= 1e-4 relative RMSE against FP64; BF16).

Workload (one step = one full fdk(plan, proj): view weights + ramp filter + cone-beam
back-projection): CtFanFlat ns=512, nt=384, ds=dt=1, dsd=1000, dso=600, na=720 over 360
deg; ImageGeom 512x512x256 at 0.5 mm; projections of 30 seeded random ellipsoids
(centres in the cylinder r<=100, |z|<=50, semi-axes U[3,60], ZYZ Euler angles, density
U[-0.3,1]) computed on the GPU.  One step is 512*512*256*720 = 48.3e9 voxel-view
updates.  Inputs (566 MB of projections) are larger than L2 (129 MB).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU (torchrun): every rank reconstructs its own scan (independent replicas,
weak scaling, no collective on the data path); the timed region is bracketed by a
barrier and the max time over ranks is reported.  `--impl reference` times the
reference algorithm's CPU restatement (the oracle port; the Julia reference cannot run
here) on the host cores for the same workload, sampled by z-slab.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sinograms.jl_gb300"))

WORKLOAD = "fdk_ctfanflat_512x512x256_from_512x384x720"
GEOM = dict(ns=512, nt=384, ds=1.0, dt=1.0, dsd=1000.0, dod=400.0, na=720, orbit=360.0)
IMG = dict(dims=(512, 512, 256), deltas=(0.5, 0.5, 0.5))
METRIC = "FDK voxel-view updates/s: plain FP32 vs BF16 form at <=1e-4 rel RMSE vs FP64"
UNIT = "voxel-view updates/s"
F_UPD = 15  # FP32 flops per voxel-view update counted for the compute roofline
FORMS = {"f32": "FP32 filtered projections (FP32 pairs (y, y[s+1] - y)), FP32 interpolation and accumulation",
         "bf16": "BF16 filtered projections, FP32 interpolation and accumulation",
         "f16": "FP16 quads of the filtered projections (y, y[t+1] - y, y[s+1] - y, mixed difference; one "
                "power-of-two scale per call), FP16 interpolation, FP32 accumulation"}
NOMINAL_FP32_TFLOPS = 152 * 128 * 2 * 2.070e9 / 1e12  # 152 SMs x 128 lanes x FMA x max clock
# Denominators used only when MEASURED_PEAKS.json is absent: one earlier GB300 measurement of a
# STREAM-style copy and of a cuBLAS bf16 GEMM burst.
FALLBACK_HBM_GBS = 6800.0
FALLBACK_BF16_TFLOPS = 1900.0


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int, device) -> float:
    """The slowest rank's value (the timing contract: max over ranks); identity when ws == 1.
    `device` holds the reduction tensor: "cuda" under NCCL, "cpu" under gloo."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(ws: int, units_per_rank: float, steps: int, max_ms: float) -> float:
    """Whole-job throughput of independent replicas: all ranks' units / the slowest rank's time."""
    return ws * units_per_rank * steps / (max_ms / 1e3)


def _phantom():
    from sinograms.phantoms import random_ellipsoids  # seeded numpy table (no library call)
    return random_ellipsoids(30, 3, 100.0, 50.0, axes=(3.0, 60.0), dens=(-0.3, 1.0))


def _config(ws: int) -> dict:
    """The workload's `config` object, the same for both arms (the arithmetic form is reported
    beside it, in `form`)."""
    return {"workload": WORKLOAD, **GEOM, "image": list(IMG["dims"]), "voxel_mm": 0.5,
            "updates_per_step": int(np.prod(IMG["dims"])) * GEOM["na"],
            "l2": "inputs larger than L2 (566 MB projections per step)", "parallelism": f"replicas x{ws}"}


def _oracle_geom():
    return dict(kind="flat", offset_s=0.0, offset_t=0.0, orbit_start=0.0, source_offset=0.0, **GEOM)


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def _issue_roofline(updates, back_ms, clocks, form):
    """The bound the back-projector actually meets: SM instruction issue.  Thread
    instructions per update come from the committed ncu capture of this kernel (storage form
    `form`) at this size; the peak is 152 SMs x 4 schedulers x 32 lanes per cycle at the sampled
    SM clock."""
    ipu = _from_profile("fdk_tma_kernel_bench_issue.md", f"thread_instructions_per_update_{form}")
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    peak = 152 * 4 * 32 * mhz * 1e6
    if ipu is None:
        return None
    achieved = ipu * updates / (back_ms / 1e3)
    return {"thread_instructions_per_update": ipu, "achieved_per_s": achieved, "peak_per_s": peak,
            "frac": achieved / peak, "source": "profiles/fdk_tma_kernel_bench_issue.md (ncu smsp__inst_executed)"}


def _bp_roofline(updates, back_ms):
    """The back-projection bound of the task's scope table: R_bp = min(P_fp32 / F_upd,
    BW_smem / B_upd), with F_upd = 15 FP32 flops and B_upd = 4 taps x 4 B from shared memory per
    update, and P_fp32, BW_smem measured on this GPU by the library's microbenchmarks.  The
    FP32 form stores (y, y[next] - y) pairs, so it actually loads one or two 8-byte pairs per
    update (one in the streaming form), not four 4-byte taps."""
    import sinograms as S
    try:
        pk = S.measure_peaks()
    except Exception as e:  # the headline line must still print
        return {"error": f"{type(e).__name__}: {e}"}
    b_upd = 16.0
    r_fp32 = pk["fp32_flops_per_s"] / F_UPD
    r_smem = pk["smem_load_bytes_per_s"] / b_upd
    achieved = updates / (back_ms / 1e3)
    return {"unit": UNIT, "flops_per_update": F_UPD, "measured_fp32_tflops": pk["fp32_flops_per_s"] / 1e12,
            "fp32_bound": r_fp32, "smem_bytes_per_update": b_upd,
            "measured_smem_load_tbs": pk["smem_load_bytes_per_s"] / 1e12, "smem_bound": r_smem,
            "smem_bytes_per_update_as_loaded": "8 (streaming form, one (y, dy) pair) to 16 (four-tap form, two pairs)",
            "r_bp": min(r_fp32, r_smem), "achieved": achieved, "frac": achieved / min(r_fp32, r_smem),
            "source": "sgb_measure_peaks (conflict-free 16-byte shared loads; 8 independent FMA chains)"}


def _filter_roofline(form, peaks):
    """Tensor-core work of the ramp filter (split-BF16 GEMM on first differences): 2 x rows x
    K x N x products, K = ns rounded up to 32, N = the output columns the MMAs compute
    (256-column blocks, the last rounded up to 16), 6 products for FP32 storage (3 pieces)
    and 3 for BF16 and F16 storage (2 pieces).  The stage time includes the split pass."""
    ns, rows = GEOM["ns"], GEOM["nt"] * GEOM["na"]
    nout = form["plan"].info()["pitch"]
    k = -(-ns // 32) * 32
    n = sum(min(256, -(-(nout - n0) // 16) * 16) for n0 in range(0, nout, 256))
    products = 6 if form["plan"].storage == "f32" else 3
    flops = 2.0 * rows * k * n * products
    achieved = flops / (form["filter_ms"] / 1e3) / 1e12
    peak = peaks.get("bf16_tflops")
    src = "MEASURED_PEAKS.json bf16_tflops (burst), of measured"
    if not peak:
        peak, src = FALLBACK_BF16_TFLOPS, "fallback 1.9 PFLOP/s bf16 burst (MEASURED_PEAKS.json absent), of fallback"
    return {"bound": "tensor", "kernel": "split_rows_kernel + filter_gemm_kernel", "achieved": achieved,
            "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "tensor_flops_per_launch": flops, "peak_source": src}


def _from_profile(name: str, key: str):
    """A figure recorded from an ncu capture in profiles/<name> (a line 'key: N'), or None."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(p):
            if line.strip().startswith(key + ":"):
                return float(line.split(":", 1)[1].split()[0])
    except Exception:
        pass
    return None



class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev_index):
        self.proc = None
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(dev_index).uuid)
            sel = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
        except Exception:
            sel = str(dev_index)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", sel], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.15)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def run_ours(args):
    import torch
    import torch.distributed as dist

    import sinograms as S

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if ws > 1:
            dist.barrier()

    rg = S.CtFanFlat(**GEOM)
    ig = S.ImageGeom(IMG["dims"], IMG["deltas"])
    nvox = int(np.prod(IMG["dims"]))
    upd = nvox * rg.na
    proj = S.ellipsoid_proj(rg, _phantom(), device=True)  # each rank: its own scan
    st = torch.cuda.current_stream()
    forms = {}
    outs = {}
    for storage in ("f32", "bf16", "f16"):
        plan = S.plan_fbp(rg, ig, storage=storage)
        plan.set_timing(True)
        img = torch.empty(tuple(reversed(IMG["dims"])), dtype=torch.float32, device="cuda")
        for _ in range(args.warmup):
            S.fdk(plan, proj, out=img, sync=False)
        torch.cuda.synchronize()
        barrier()
        sampler = ClockSampler(local)
        l0 = S.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        fms, bms = [], []
        for _ in range(args.steps):
            S.fdk(plan, proj, out=img, sync=False)
            f_ms, b_ms = plan.last_timing()
            fms.append(f_ms)
            bms.append(b_ms)
        e1.record(st)
        torch.cuda.synchronize()
        launches = S.launch_count() - l0
        clocks = sampler.stop()
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1), ws, "cuda")
        forms[storage] = dict(ms_per_step=ms / args.steps, value=replica_throughput(ws, upd, args.steps, ms),
                              filter_ms=float(np.mean(fms)), back_ms=float(np.mean(bms)), gpu_launches=launches,
                              clocks=clocks, plan=plan)
        outs[storage] = img
    # headline: the F16 storage form, the fastest form within the metric's 1e-4 relative RMSE
    # against FP64 on this workload (the accuracy leg below measures every form in the same run,
    # `forms.*.meets_1e-4`; tests/test_gpu_full_size.py holds it to 1e-4).  The FP32 form (plain) and
    # the BF16 form (1.8e-4, misses the bound) are reported beside it.
    head = "f16"
    # e2e through the public API with pinned host buffers: every step copies its projections
    # in (566 MB) and its volume out (268 MB).  Steps rotate over three plans on three streams,
    # as a scan-after-scan user would run them, so a step's copies overlap the others'
    # back-projections with two steps of slack; the wall clock spans all steps and the final
    # synchronisation.
    nplan = 3
    plans = [forms[head]["plan"]] + [S.plan_fbp(rg, ig, storage=head) for _ in range(nplan - 1)]
    plans[0].set_timing(False)  # a user's call: no stage-timing events
    streams = [torch.cuda.Stream() for _ in range(nplan)]
    hproj = torch.empty(proj.shape, dtype=torch.float32, pin_memory=True)
    hproj.copy_(proj)
    hp = hproj.numpy()
    himg_t = [torch.empty(tuple(reversed(IMG["dims"])), dtype=torch.float32, pin_memory=True) for _ in range(nplan)]
    himgs = [t.numpy() for t in himg_t]
    # the host link's copy rates in this run (pinned buffers, one 566 MB / 268 MB copy each)
    copy_gbs = {}
    dimg = torch.empty(tuple(reversed(IMG["dims"])), dtype=torch.float32, device="cuda")
    for name, fn, nbytes in (("h2d", lambda: proj.copy_(hproj, non_blocking=True), proj.numel() * 4),
                             ("d2h", lambda: himg_t[0].copy_(dimg, non_blocking=True), nvox * 4)):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        copy_gbs[name] = nbytes / (time.perf_counter() - t0) / 1e9
    del dimg
    for i in range(nplan):  # warm every plan (staging buffers allocated)
        S.fdk(plans[i], hp, out=himgs[i])
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(streams[k % nplan]):
            S.fdk(plans[k % nplan], hp, out=himgs[k % nplan], sync=False)
    for i in range(nplan):
        with torch.cuda.stream(streams[i]):
            plans[i].sync()
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws, "cuda")
    barrier()
    # the same public call on one plan and one stream, each step waiting for its volume: the
    # copies do not overlap any compute
    t0 = time.perf_counter()
    for k in range(args.steps):
        S.fdk(plans[0], hp, out=himgs[0])
    e2e_1s = max_over_ranks(time.perf_counter() - t0, ws, "cuda")
    barrier()
    ref_vol = outs[head].cpu().numpy()
    tol = 1e-6 * float(outs[head].abs().max())
    # himgs[1]: a pipelined step's volume; himgs[0]: the single-stream run's
    e2e_ok = all(bool(np.allclose(h, ref_vol, rtol=0, atol=tol)) for h in (himgs[0], himgs[1]))

    peaks = _peaks()
    hbm = peaks.get("hbm_gbs")
    hbm_src = "MEASURED_PEAKS.json hbm_gbs (burst copy), of measured"
    if not hbm:
        hbm, hbm_src = FALLBACK_HBM_GBS, "fallback 6.8 TB/s (MEASURED_PEAKS.json absent), of fallback"
    f = forms[head]
    # read the filtered projections once (2 B per sample for the 16-bit forms) + write the volume
    alg_bytes = proj.numel() * (4 if head == "f32" else 2) + nvox * 4
    achieved = alg_bytes / (f["back_ms"] / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": f["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": f["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": head,
        "data": "synthetic: 30 seeded random ellipsoids, analytic cone-beam projections generated on the GPU",
        "config": _config(ws),
        "form": {"storage": head, "description": FORMS[head]},
        "forms": {k: {"value": v["value"], "ms_per_step": v["ms_per_step"], "filter_ms": v["filter_ms"],
                      "back_ms": v["back_ms"], "vs_f32": v["value"] / forms["f32"]["value"],
                      "plan": v["plan"].info()} for k, v in forms.items()},
        "e2e": {"value": replica_throughput(ws, upd, args.steps, e2e_s * 1e3), "unit": UNIT,
                "h2d_bytes_per_step": proj.numel() * 4, "d2h_bytes_per_step": nvox * 4,
                "ms_per_step": e2e_s * 1e3 / args.steps,
                "pipeline": "fdk(plan, host proj) with pinned buffers; steps rotate over three plans on three "
                            "streams, so a step's copies overlap the others' compute",
                "copy_gbs": copy_gbs,
                "volume_matches_device_run": e2e_ok,
                "single_stream": {"value": replica_throughput(ws, upd, args.steps, e2e_1s * 1e3),
                                  "ms_per_step": e2e_1s * 1e3 / args.steps,
                                  "pipeline": "fdk(plan, host proj, out=host volume) on one plan and one stream, "
                                              "synchronous: copies in, filter, back-projection, copy out"}},
        "roofline": {"bound": "hbm", "kernel": "fdk_tma_kernel", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "peak_source": hbm_src,
                     "alg_bytes_per_launch": alg_bytes,
                     "traffic": _from_profile("fdk_tma_kernel_bench_dram.md", f"traffic_bytes_per_launch_{head}"),
                     "issue": _issue_roofline(upd, f["back_ms"], f["clocks"], head),
                     "fp32_issue": {"flops_per_update": F_UPD,
                                    "achieved_tflops": F_UPD * upd / (f["back_ms"] / 1e3) / 1e12,
                                    "peak_tflops_nominal": NOMINAL_FP32_TFLOPS,
                                    "frac": F_UPD * upd / (f["back_ms"] / 1e3) / 1e12 / NOMINAL_FP32_TFLOPS}},
        "bp_roofline": _bp_roofline(upd, f["back_ms"]),
        "filter_roofline": _filter_roofline(forms[head], peaks),
        "plan": forms[head]["plan"].info(),
        "gpu_launches": f["gpu_launches"],
        "clocks": f["clocks"],
    }
    # the side measurements below record their error instead of losing the headline line
    if not args.no_batch:
        try:
            line["batched"] = measure_batched(args)
        except Exception as e:
            line["batched"] = {"error": f"{type(e).__name__}: {e}"}
        for form in ("f16", "bf16"):
            try:
                b = measure_batched(args, storage=form, rerun_check=False)
                line["batched"].setdefault("forms", {})[form] = {
                    k: b[k] for k in ("value", "ms_per_run", "stage_ms", "box_classes", "back_updates_per_s_by_class")}
            except Exception as e:
                line["batched"].setdefault("forms", {})[form] = {"error": f"{type(e).__name__}: {e}"}
    if not args.no_2d:
        line["configs_2d"] = measure_2d(args)
        line["configs_2d"]["sf_pair_arc_888x90"] = measure_sf(args)
    if ws == 1 and rank == 0 and not args.no_cpu:
        try:
            base, acc = cpu_leg({k: v.cpu().numpy() for k, v in outs.items()}, proj.cpu().numpy())
            line["cpu_baseline"] = base
            line["accuracy_vs_fp64"] = acc
            for k_ in line["forms"]:
                line["forms"][k_]["meets_1e-4"] = bool(acc[k_]["rel_rmse"] <= 1e-4)
        except Exception as e:
            line["cpu_baseline"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def measure_batched(args, storage: str = "f32", rerun_check: bool = True):
    """Batched FDK workload: 48 seeded CBCT scans of uneven size (volumes 128^3 .. 384x384x256,
    na 180..720, ns 256..768, nt 128..384, flat/arc) reconstructed by one CUDA graph with one
    persistent back-projection launch per box class; `storage` form of the filtered
    projections.  Device-resident inputs."""
    import torch

    import sinograms as S
    rgs, igs, ells = S.random_ct_scans(48, 4)
    t0 = time.perf_counter()
    batch = S.FDKBatch(rgs, igs, storage=storage)
    t_plan = time.perf_counter() - t0
    projs = []
    for i, (rg, e) in enumerate(zip(rgs, ells)):
        projs.append(S.ellipsoid_proj(rg, e, device=True))
        batch.set_input(i, projs[-1])
    st = torch.cuda.current_stream()
    for _ in range(args.warmup):
        batch.run(sync=False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = S.launch_count()
    e0.record(st)
    for _ in range(args.steps):
        batch.run(sync=False)
    e1.record(st)
    torch.cuda.synchronize()
    batch.run()  # synchronous run: checks the kernel's error flags
    ms = e0.elapsed_time(e1) / args.steps
    info = batch.info()
    stages = batch.timing()
    # every persistent launch does its work on every run: with all inputs doubled, every scan's
    # volume must come out exactly doubled (scaling by 2 is exact in every stage)
    doubled = None
    if rerun_check:
        first = [batch.get_output(i, device=True) for i in range(len(rgs))]
        for i, p in enumerate(projs):
            batch.set_input(i, 2 * p)
        batch.run()
        doubled = all(bool(torch.equal(batch.get_output(i, device=True), 2 * first[i])) for i in range(len(rgs)))
        del first
    del projs, batch
    return {"workload": "fdk_batch_48_uneven_scans_seed4", "storage": storage, "value": info["updates"] / (ms / 1e3),
            "unit": UNIT,
            "ms_per_run": ms, "updates_per_run": info["updates"], "scans": info["scans"],
            "work_items": info["work_items"], "persistent_ctas": info["ctas"], "persistent_launches": info["launches"],
            "plan_seconds": t_plan, "gpu_launches_per_run": (S.launch_count() - l0) / args.steps,
            "stage_ms": {"filters": stages[0], "back_by_box_class": stages[1:]}, "box_classes": info["classes"],
            "back_updates_per_s_by_class": [c["mupdates"] * 1e6 / (t / 1e3) if t > 0 else None
                                            for c, t in zip(info["classes"], stages[1:])],
            "rerun_with_doubled_inputs_exact": doubled}


def _per_call_ms(fn, reps):
    """Device time per call of fn (enqueued back to back on the current stream)."""
    import torch
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


def _accuracy_2d(out, g, igd, sino, window, rfov):
    """Relative RMSE and max error of a 2D FBP against the FP64 oracle on the same FP32
    sinogram: over the FOV disk less 1 mm (the image corners meet the detector edge, where FP32
    and FP64 rounding decide the whole-tap rule differently) and over the whole image."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    ref = O.fbp(g, igd, sino, shape=window)
    nx, ny = igd["dims"]
    dx, dy = igd["deltas"]
    x = dx * (np.arange(nx) - (nx - 1) / 2)
    y = dy * (np.arange(ny) - (ny - 1) / 2)
    inside = (x[None, :] ** 2 + y[:, None] ** 2) <= (rfov - 1.0) ** 2
    return {"rel_rmse_fov": O.rel_rmse(out[inside], ref[inside]),
            "max_abs_err_rel_fov": float(np.abs(out - ref)[inside].max() / np.abs(ref).max()),
            "rel_rmse_image": O.rel_rmse(out, ref), "oracle": "FP64 C restatement, same FP32 sinogram"}


def measure_2d(args):
    """The 2D workloads beside the headline, device-resident, on seeded synthetic inputs:
    SinoPar 256 x 180 -> 256^2 with a Hann window; SinoFanArc 888 x 512 views over a short scan ->
    512^2 (Parker weights, 0.5% noise); and the learned row filter's sparse-view scan (SinoFanArc
    888 x 90 views over 360 deg -> 512^2): plain FBP against FBP with the CNN row filter and with
    the learned linear (ramp) filter, time and image RMSE against the phantom on 8 held-out scans;
    the data come from the arc-detector distance-driven projector."""
    import torch

    import sinograms as S
    from sinograms import learned as LF
    reps = max(args.steps, 20)
    out = {}
    try:
        rg = S.SinoPar(nb=256, d=1.0, na=180, orbit=180.0)
        plan = S.plan_fbp(rg, S.ImageGeom((256, 256), (1.0, 1.0)), window=S.Window("hann"))
        sino = S.ellipse_sino(rg, S.random_ellipses(10, 1, 100.0), device=True)
        ms = _per_call_ms(lambda: S.fbp(plan, sino, sync=False), reps)
        plan.set_timing(True)
        S.fbp(plan, sino)
        f_ms, b_ms = plan.last_timing()
        plan.set_timing(False)
        out["par_256x180_hann"] = {"ms_per_fbp": ms, "filter_ms": f_ms, "back_ms": b_ms,
                                   "back_updates_per_s": 256 * 256 * 180 / (b_ms / 1e3)}
        if not args.no_cpu:
            g = dict(kind="par", nb=256, d=1.0, offset=0.0, na=180, orbit=180.0, orbit_start=0.0)
            out["par_256x180_hann"]["accuracy_vs_fp64"] = _accuracy_2d(
                S.fbp(plan, sino).cpu().numpy(), g, dict(dims=(256, 256), deltas=(1.0, 1.0)),
                sino.cpu().numpy(), "hann", S._rfov(rg))
        base = S.SinoFanArc(nb=888, d=1.0239, dsd=949.075, dod=408.075, na=2, orbit=360.0)
        orbit = 180.0 + 2.0 * float(np.degrees(S._gamma_max(base)))  # short scan: 180 deg + fan angle
        rg = S.SinoFanArc(nb=888, d=1.0239, dsd=949.075, dod=408.075, na=512, orbit=orbit)
        plan = S.plan_fbp(rg, S.ImageGeom((512, 512), (0.9766, 0.9766)))
        sino = S.ellipse_sino(rg, S.random_ellipses(20, 2, 220.0, axes=(4.0, 120.0), dens=(-0.3, 1.0)), device=True)
        g = torch.Generator(device="cuda").manual_seed(102)
        sino = sino + 0.005 * sino.abs().max() * torch.randn(sino.shape, device="cuda", generator=g)
        ms = _per_call_ms(lambda: S.fbp(plan, sino, sync=False), reps)
        plan.set_timing(True)
        S.fbp(plan, sino)
        f_ms, b_ms = plan.last_timing()
        plan.set_timing(False)
        out["arc_888x512_short_scan"] = {"ms_per_fbp": ms, "filter_ms": f_ms, "back_ms": b_ms,
                                         "back_updates_per_s": 512 * 512 * 512 / (b_ms / 1e3)}
        if not args.no_cpu:
            g = dict(kind="arc", nb=888, d=1.0239, offset=0.0, dsd=949.075, dod=408.075, source_offset=0.0,
                     orbit_start=0.0, na=512, orbit=orbit)
            out["arc_888x512_short_scan"]["accuracy_vs_fp64"] = _accuracy_2d(
                S.fbp(plan, sino).cpu().numpy(), g, dict(dims=(512, 512), deltas=(0.9766, 0.9766)),
                sino.cpu().numpy(), "none", S._rfov(rg))
        rg, ig = LF.sparse_fan_geometry()
        plan = S.plan_fbp(rg, ig)
        lf = LF.LearnedFilter.load(LF.default_weights_path())
        geo = S.BddGeo.from_geoms(rg, ig)
        mask = torch.as_tensor(ig.mask, device="cuda")
        gen = torch.Generator(device="cuda").manual_seed(900000)
        ramp = LF.LearnedRamp.load(LF.default_ramp_path())
        plan_ramp = ramp.plan(rg, ig)
        rp, rl, rr, kept, kept_r = [], [], [], 0, 0
        for i in range(8):
            img = LF.ellipse_image(ig.with_mask(None), LF.phantom_ellipses(900000 + i))
            s = LF.dd_project(img, geo)
            s = s + 0.005 * s.abs().max() * torch.randn(s.shape, device="cuda", generator=gen)
            rp.append(float((S.fbp(plan, s) - img)[mask].pow(2).mean().sqrt()))
            rr.append(float((S.fbp(plan_ramp, s) - img)[mask].pow(2).mean().sqrt()))
            kept_r += int(LF.fbp_learned_ramp(plan_ramp, plan, s)[1]["used"] == "learned")
            im_l, info = LF.fbp_learned(plan, lf, s, judge=True)
            rl.append(float((LF.fbp_backproject(plan, lf.apply(LF.fbp_filter_rows(plan, s))) - img)[mask]
                            .pow(2).mean().sqrt()))
            kept += int(info["used"] == "learned")
        s = s.contiguous()
        ms_plain = _per_call_ms(lambda: S.fbp(plan, s, sync=False), reps)
        ms_ramp = _per_call_ms(lambda: S.fbp(plan_ramp, s, sync=False), reps)
        ms_learned = _per_call_ms(lambda: LF.fbp_backproject(
            plan, lf.apply(LF.fbp_filter_rows(plan, s, sync=False), sync=False), sync=False), reps)
        z = LF.fbp_filter_rows(plan, s)
        ms_net = _per_call_ms(lambda: lf.apply(z, sync=False), reps)
        # forward FLOPs: 2 per multiply-add over the 5 layers (1->32, 3 x 32->32, 32->1, kernel 9)
        net_flops = 2.0 * z.numel() * 9 * (32 + 3 * 32 * 32 + 32)
        # distance-driven projection of a 512^2 image over the scan's 90 views; FLOPs per the fixed
        # count na * nPix * (2 nPix + 7 (nDet + 1))
        img0 = LF.ellipse_image(ig.with_mask(None), LF.phantom_ellipses(900000))
        dd_plan, ph0 = LF.bdd_plan(geo), LF.image_to_dd(img0)
        sino_dd = torch.empty((geo.nDet, len(geo.angle)), device="cuda")
        img_dd = torch.empty_like(ph0)
        ms_dd = _per_call_ms(lambda: dd_plan.project(ph0, out=sino_dd, sync=False), reps)
        ms_ddb = _per_call_ms(lambda: dd_plan.backproject(sino_dd, out=img_dd, sync=False), reps)
        dd_flops = float(len(geo.angle) * geo.nPix * (2 * geo.nPix + 7 * (geo.nDet + 1)))
        try:
            fp32_peak = S.measure_peaks()["fp32_flops_per_s"]
        except Exception:
            fp32_peak = None
        out["learned_filter_arc_888x90"] = {
            "ms_plain_fbp": ms_plain, "ms_learned_fbp": ms_learned, "ms_network": ms_net,
            "network_tflops": net_flops / (ms_net / 1e3) / 1e12,
            "network_frac_of_bf16_peak": net_flops / (ms_net / 1e3) / ((_peaks().get("bf16_tflops") or FALLBACK_BF16_TFLOPS) * 1e12),
            "dd_project_ms": ms_dd, "dd_backproject_ms": ms_ddb,
            "dd_project_call": "BddPlan calls on device tensors, enqueued back to back: project = output clear +"
                               " one launch; backproject = output clear + per-view set-up + one launch",
            "dd_project_tflops": dd_flops / (ms_dd / 1e3) / 1e12,
            "dd_project_frac_of_fp32": (dd_flops / (ms_dd / 1e3) / fp32_peak) if fp32_peak else None,
            "rmse_vs_phantom_plain": float(np.mean(rp)), "rmse_vs_phantom_learned": float(np.mean(rl)),
            "judge_kept_learned": f"{kept}/8", "weights": os.path.basename(LF.default_weights_path()),
            "ms_learned_ramp_fbp": ms_ramp, "rmse_vs_phantom_learned_ramp": float(np.mean(rr)),
            "judge_kept_learned_ramp": f"{kept_r}/8", "ramp_gain": os.path.basename(LF.default_ramp_path())}
        ms_train, _ = _lf_train_step_ms(10)
        out["learned_filter_arc_888x90"]["train_step_ms"] = ms_train
        out["learned_filter_arc_888x90"]["train_step"] = ("LearnedFilter.train_step on 4096 rows x 888 (forward, "
                                                          "backward, Adam), CUDA-synchronised wall time, mean of 10")
    except Exception as e:  # the headline line must still print
        out["error"] = f"{type(e).__name__}: {e}"
    return out


# --------------------------------------------------------------------- CPU side

def _slab_rows(rg, z_lo, z_hi, rxy):
    """Detector rows (0-based, inclusive) that voxels with z in [z_lo, z_hi] and
    radius <= rxy can reach: t' = mag * z with mag in [dsd/(dso+rxy), dsd/(dso-rxy)]."""
    dso = rg["dsd"] - rg["dod"]
    mags = (rg["dsd"] / (dso + rxy), rg["dsd"] / (dso - rxy))
    ts = [m * z / rg["dt"] for m in mags for z in (z_lo, z_hi)]
    wt = (rg["nt"] + 1) / 2
    lo = max(0, int(math.floor(min(ts) + wt)) - 2 - 1)
    hi = min(rg["nt"] - 1, int(math.floor(max(ts) + wt)) + 2)
    return lo, hi


def cpu_fdk_slab(O, proj, rg, z_idx, threads, bits=32):
    """Reference algorithm on the CPU for the voxels in z-slices z_idx: weight, FFT ramp
    filter of the detector rows those voxels reach, back-projection. Returns
    (image_slab, seconds, updates)."""
    ax = O.image_axes(dict(dims=IMG["dims"], deltas=IMG["deltas"]))
    zc = ax[2][z_idx]
    rxy = math.hypot(abs(ax[0]).max(), abs(ax[1]).max())
    lo, hi = _slab_rows(rg, zc.min(), zc.max(), rxy)
    dt_ = np.float32 if bits == 32 else np.float64
    t0 = time.perf_counter()
    w = O.fdk_weights(rg)[:, lo:hi + 1, :].astype(dt_)
    band = proj[:, lo:hi + 1, :].astype(dt_) * w
    Hk = O.fbp_filter(rg)
    filt = np.zeros(proj.shape, dtype=dt_)
    filt[:, lo:hi + 1, :] = O.sino_filter_fft(band, Hk, workers=threads)
    img = _back_z(O, filt, rg, ax, zc, bits)
    sec = time.perf_counter() - t0
    return img, sec, IMG["dims"][0] * IMG["dims"][1] * len(z_idx) * rg["na"]


def _back_z(O, filt, rg, ax, zc, bits, xs=None, ys=None):
    import ctypes
    L = O.lib(bits)
    xc = np.ascontiguousarray(ax[0] if xs is None else ax[0][xs])
    yc = np.ascontiguousarray(ax[1] if ys is None else ax[1][ys])
    zc = np.ascontiguousarray(zc)
    na, nt, ns = filt.shape
    img = np.zeros((len(zc), len(yc), len(xc)), dtype=filt.dtype)
    b = np.ascontiguousarray(O.ar(rg))
    rc = L.orc_cbct_back(ctypes.c_void_p(img.ctypes.data), ctypes.c_void_p(filt.ctypes.data), ns, nt, na,
                         ctypes.c_void_p(b.ctypes.data), ctypes.c_double(rg["dsd"]), ctypes.c_double(O.dso(rg)),
                         ctypes.c_double(rg["ds"]), ctypes.c_double(rg["dt"]), ctypes.c_float(0.0),
                         ctypes.c_float(0.0), 0, ctypes.c_void_p(xc.ctypes.data), ctypes.c_void_p(yc.ctypes.data),
                         ctypes.c_void_p(zc.ctypes.data), len(xc), len(yc), len(zc), None, 1)
    assert rc == 0
    return img


def _threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def cpu_leg(gpu_imgs, proj):
    """CPU baseline (FP32 restatement of the reference loops, all host threads) on a
    central z-slab, and FP64 accuracy of both GPU forms on a sparse voxel sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    rg = _oracle_geom()
    th = _threads()
    nz = IMG["dims"][2]
    # calibrate on 2 slices, then size the slab for ~10 s of CPU work
    _, sec, u = cpu_fdk_slab(O, proj, rg, np.arange(nz // 2 - 1, nz // 2 + 1), th)
    k = int(min(64, max(4, 2 * 10.0 / max(sec, 1e-3))))
    z_idx = np.arange(nz // 2 - k // 2, nz // 2 - k // 2 + k)
    _, sec, u = cpu_fdk_slab(O, proj, rg, z_idx, th)
    base = {"value": u / sec, "unit": UNIT, "cores": th, "kind": "port",
            "sample": f"fdk of the central {k}-slice z-slab (512x512x{k} voxels x 720 views = {u:.3g} updates): "
                      f"weights + FFT ramp filter of the detector rows the slab reaches + FP32 back-projection "
                      f"(oracle restatement of the reference loops; Julia is not available here)",
            "seconds": sec}
    # FP64 accuracy on a sparse sample: every 16th x/y voxel, 8 z-slices spread over z
    xs, ys = np.arange(0, 512, 16), np.arange(0, 512, 16)
    zs = np.linspace(0, nz - 1, 8).round().astype(int)
    filt = O.sino_filter_fft(proj.astype(np.float64) * O.fdk_weights(rg), O.fbp_filter(rg), workers=th)
    ax = O.image_axes(dict(dims=IMG["dims"], deltas=IMG["deltas"]))
    ref = _back_z(O, filt, rg, ax, ax[2][zs], 64, xs, ys)
    acc = {}
    for k_, img in gpu_imgs.items():
        sub = img[np.ix_(zs, ys, xs)]
        acc[k_] = {"rel_rmse": O.rel_rmse(sub, ref),
                   "max_abs_err_rel": float(np.abs(sub - ref).max() / np.abs(ref).max()),
                   "sample": "32x32x8 voxels (every 16th x,y; 8 z-slices), FP64 oracle"}
    return base, acc


def run_reference(args):
    """Reference arm: the reference algorithm on the host cores (oracle FP32 port), same
    metric and workload; each step is a bounded z-slab sample."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    rg = _oracle_geom()
    th = _threads()
    nz = IMG["dims"][2]
    k = 8
    slabs = [np.arange(z0, z0 + k) for z0 in range(0, nz, k)]
    used = [slabs[i % len(slabs)] for i in range(args.warmup)]
    used += [slabs[(args.warmup + i * 5) % len(slabs)] for i in range(args.steps)]
    # projections of the same phantom by the oracle's CPU projector (this arm runs no GPU code),
    # on the detector rows the sampled slabs reach
    ax = O.image_axes(dict(dims=IMG["dims"], deltas=IMG["deltas"]))
    rxy = math.hypot(abs(ax[0]).max(), abs(ax[1]).max())
    rows = set()
    for zi in used:
        lo, hi = _slab_rows(rg, ax[2][zi].min(), ax[2][zi].max(), rxy)
        rows.update(range(lo, hi + 1))
    proj = O.ellipsoid_proj(rg, _phantom(), rows=sorted(rows)).astype(np.float32)
    for zi in used[:args.warmup]:
        cpu_fdk_slab(O, proj, rg, zi, th)
    tot_s, tot_u = 0.0, 0
    for zi in used[args.warmup:]:
        _, sec, u = cpu_fdk_slab(O, proj, rg, zi, th)
        tot_s += sec
        tot_u += u
    v = tot_u / tot_s
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot_s / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "impl": "reference",
            "data": "synthetic: 30 seeded random ellipsoids (same phantom as the GPU arm), projected by the "
                    "oracle's CPU projector on the detector rows the sampled slabs reach",
            "config": _config(ws),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": th, "kind": "port",
                             "sample": f"each step: fdk of one {k}-slice z-slab (512x512x{k} x 720 views): weights + "
                                       "FFT ramp filter of the rows it reaches + FP32 back-projection; oracle "
                                       "restatement of the reference (Julia not available)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batch_case(args):
    """Profiling case for the batched workload: build the 48-scan batch, run it twice."""
    import torch

    import sinograms as S
    rgs, igs, ells = S.random_ct_scans(48, 4)
    batch = S.FDKBatch(rgs, igs)
    for i, (rg, e) in enumerate(zip(rgs, ells)):
        batch.set_input(i, S.ellipsoid_proj(rg, e, device=True))
    for _ in range(2):
        batch.run()
    torch.cuda.synchronize()
    print(json.dumps({"case": "fdk_batch_48_uneven_scans_seed4", **batch.info(), "stage_ms": batch.timing()}))


def run_dd_case(args):
    """Distance-driven projector pair on the learned-filter scan (512^2 image, 888 bins on the arc
    detector, 90 views): one random-ellipse phantom projected and back-projected through its
    BddPlan, 5 + 20 times each, device tensors, calls enqueued back to back."""
    import torch

    import sinograms as S
    from sinograms import learned as LF
    rg, ig = LF.sparse_fan_geometry()
    geo = S.BddGeo.from_geoms(rg, ig)
    plan = LF.bdd_plan(geo)
    ph = LF.image_to_dd(LF.ellipse_image(ig.with_mask(None), LF.phantom_ellipses(900000)))
    sino = torch.empty((geo.nDet, len(geo.angle)), device="cuda")
    back = torch.empty_like(ph)
    ms = {}
    for name, fn in (("project", lambda: plan.project(ph, out=sino, sync=False)),
                     ("backproject", lambda: plan.backproject(sino, out=back, sync=False))):
        for _ in range(5):
            fn()
        ms[name] = _per_call_ms(fn, 20)
    print(json.dumps({"case": "dd_fanarc_512x512_888x90", "ms_project": ms["project"],
                      "ms_backproject": ms["backproject"], "sino_sum": float(sino.sum())}))


def _sf_setup():
    """Separable-footprint pair on the learned-filter scan geometry (SinoFanArc 888 x 90 over 360 deg,
    512^2 at 0.9766 mm, no mask), its plan and one seeded random-ellipse phantom on the device."""
    import torch

    import sinograms as S
    from sinograms import learned as LF
    rg, ig = LF.sparse_fan_geometry()
    ig = ig.with_mask(None)
    plan = S.SFPlan(rg, ig)
    img = LF.ellipse_image(ig, LF.phantom_ellipses(900000))
    sino = torch.empty((rg.na, rg.nb), device="cuda")
    back = torch.empty_like(img)
    return rg, ig, plan, img, sino, back


def run_sf_case(args):
    """Separable-footprint projector pair (SinoFanArc 888 x 90, 512^2): project and back-project one
    random-ellipse phantom through its SFPlan, 5 + 20 times each, device tensors, calls enqueued back
    to back."""
    rg, ig, plan, img, sino, back = _sf_setup()
    ms = {}
    for name, fn in (("project", lambda: plan.project(img, out=sino, sync=False)),
                     ("backproject", lambda: plan.backproject(sino, out=back, sync=False))):
        for _ in range(5):
            fn()
        ms[name] = _per_call_ms(fn, 20)
    print(json.dumps({"case": "sf_fanarc_512x512_888x90", "ms_project": ms["project"],
                      "ms_backproject": ms["backproject"], "sino_sum": float(sino.sum())}))


def measure_sf(args):
    """SF pair block of the bench line: times per call, (pixel, view) pairs per second, and the
    accuracy of the SF and DD models against the analytic sinogram of the same phantom."""
    import sinograms as S
    from sinograms import learned as LF
    reps = max(args.steps, 20)
    out = {}
    try:
        rg, ig, plan, img, sino, back = _sf_setup()
        ms_p = _per_call_ms(lambda: plan.project(img, out=sino, sync=False), reps)
        ms_b = _per_call_ms(lambda: plan.backproject(sino, out=back, sync=False), reps)
        pairs = float(rg.na) * ig.dims[0] * ig.dims[1]
        ell = LF.phantom_ellipses(900000)
        ref = S.ellipse_sino(rg, ell, device=True)
        plan.project(img, out=sino)
        e_sf = float(((sino - ref).pow(2).mean() / ref.pow(2).mean()).sqrt())
        dd = LF.dd_project(img, S.BddGeo.from_geoms(rg, ig))
        e_dd = float(((dd - ref).pow(2).mean() / ref.pow(2).mean()).sqrt())
        out = {"ms_project": ms_p, "ms_backproject": ms_b,
               "project_pixel_views_per_s": pairs / (ms_p / 1e3),
               "backproject_pixel_views_per_s": pairs / (ms_b / 1e3),
               "rel_rmse_vs_analytic_sf": e_sf, "rel_rmse_vs_analytic_dd": e_dd,
               "call": "SFPlan calls on device tensors, enqueued back to back (one launch each)",
               # both kernels are bound by instruction issue (ncu issue-active of each, one launch)
               "roofline": {"bound": "issue",
                            "project_issue_active": _from_profile("sf_kernels_fanarc888_90v.md",
                                                                  "sf_project_issue_active"),
                            "backproject_issue_active": _from_profile("sf_kernels_fanarc888_90v.md",
                                                                      "sf_back_issue_active"),
                            "source": "profiles/sf_kernels_fanarc888_90v.md (ncu smsp__issue_active)"}}
    except Exception as e:  # the headline line must still print
        out["error"] = f"{type(e).__name__}: {e}"
    return out


def _lf_train_step_ms(steps):
    """Training step of the learned filter at the training script's batch: 4096 seeded rows of a
    64-scan training set of the SinoFanArc 888 x 90 workload (888 samples per row), 3 + `steps`
    calls of LearnedFilter.train_step; (CUDA-synchronised wall time per step in ms, last loss)."""
    import torch

    from sinograms import learned as LF
    rg, ig = LF.sparse_fan_geometry()
    zn, zc = LF.make_dataset(64, seed=3, rg=rg, ig=ig)
    scale = float(zc.pow(2).mean().sqrt())
    lf = LF.LearnedFilter(scale=scale, seed=1)
    idx = torch.randperm(zn.shape[0], device="cuda", generator=torch.Generator(device="cuda").manual_seed(0))[:4096]
    a, b = zn[idx].contiguous(), zc[idx].contiguous()
    for _ in range(3):
        lf.train_step(a, b, 1e-3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        loss = lf.train_step(a, b, 1e-3)
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / steps * 1e3, float(loss)


def run_lf_train_case(args):
    """The learned filter's training step (see _lf_train_step_ms), --steps timed calls."""
    ms, loss = _lf_train_step_ms(args.steps)
    print(json.dumps({"case": "lf_train_arc888x90_4096rows", "train_step_ms": ms, "rows": 4096, "L": 888,
                      "steps": args.steps, "loss": loss}))


def run_lf_apply_case(args):
    """Learned-filter inference on the 90-view scan: the plan's ramp-filtered rows of one seeded
    phantom's noisy DD sinogram, then 3 + --steps calls of LearnedFilter.apply (one lf_tc_fused
    launch each) enqueued back to back; mean time per call from CUDA events."""
    import torch

    import sinograms as S
    from sinograms import learned as LF
    rg, ig = LF.sparse_fan_geometry()
    plan = S.plan_fbp(rg, ig)
    lf = LF.LearnedFilter.load(LF.default_weights_path())
    img = LF.ellipse_image(ig.with_mask(None), LF.phantom_ellipses(900000))
    sino = LF.dd_project(img, S.BddGeo.from_geoms(rg, ig))
    sino = sino + 0.005 * sino.abs().max() * torch.randn(sino.shape, device="cuda",
                                                         generator=torch.Generator(device="cuda").manual_seed(7))
    z = LF.fbp_filter_rows(plan, sino)
    for _ in range(3):
        lf.apply(z, sync=False)
    ms = _per_call_ms(lambda: lf.apply(z, sync=False), args.steps)
    print(json.dumps({"case": "lf_apply_arc888x90", "rows": int(z.shape[0]), "L": int(z.shape[1]),
                      "ms_network": ms}))


def run_fbp2d_case(args):
    """The three 2D workloads for a back-projector capture: SinoPar 256 x 180 -> 256^2 (Hann),
    SinoFanArc 888 x 90 views -> 512^2 (the learned-filter scan) and SinoFanArc 888 x 512 views
    over a short scan -> 512^2, each planned once, then three passes of one fbp(plan, sino) per
    workload in that order (three back2_kernel launches per pass)."""
    import torch

    import sinograms as S
    from sinograms import learned as LF
    cases = []
    rg = S.SinoPar(nb=256, d=1.0, na=180, orbit=180.0)
    cases.append((S.plan_fbp(rg, S.ImageGeom((256, 256), (1.0, 1.0)), window=S.Window("hann")),
                  S.ellipse_sino(rg, S.random_ellipses(10, 1, 100.0), device=True)))
    rg, ig = LF.sparse_fan_geometry()
    cases.append((S.plan_fbp(rg, ig), S.ellipse_sino(rg, LF.phantom_ellipses(900000), device=True)))
    base = S.SinoFanArc(nb=888, d=1.0239, dsd=949.075, dod=408.075, na=2, orbit=360.0)
    orbit = 180.0 + 2.0 * float(np.degrees(S._gamma_max(base)))
    rg = S.SinoFanArc(nb=888, d=1.0239, dsd=949.075, dod=408.075, na=512, orbit=orbit)
    cases.append((S.plan_fbp(rg, S.ImageGeom((512, 512), (0.9766, 0.9766))),
                  S.ellipse_sino(rg, S.random_ellipses(20, 2, 220.0, axes=(4.0, 120.0), dens=(-0.3, 1.0)),
                                 device=True)))
    sums = []
    for _ in range(3):
        sums = [float(S.fbp(plan, sino).sum()) for plan, sino in cases]
    torch.cuda.synchronize()
    print(json.dumps({"case": "fbp2d_par256x180_arc888x90_arc888x512", "image_sums": sums}))


def run_case(args):
    """Reduced profiling case (one GPU, a few launches): fdk of 512x512x64 voxels from
    180 views of the benchmark geometry; the filtered projections (141 MB) exceed L2."""
    import torch

    import sinograms as S
    if args.case == "fdk-batch":
        return run_batch_case(args)
    if args.case == "dd-fan-888x90":
        return run_dd_case(args)
    if args.case == "fbp-2d":
        return run_fbp2d_case(args)
    if args.case == "lf-train":
        return run_lf_train_case(args)
    if args.case == "lf-apply":
        return run_lf_apply_case(args)
    if args.case == "sf-fan-888x90":
        return run_sf_case(args)
    g = dict(GEOM, na=180)
    rg = S.CtFanFlat(**g)
    ig = S.ImageGeom((512, 512, 64), IMG["deltas"])
    proj = S.ellipsoid_proj(rg, _phantom(), device=True)
    plan = S.plan_fbp(rg, ig, storage=args.storage)
    img = torch.empty((64, 512, 512), device="cuda")
    for _ in range(2):
        S.fdk(plan, proj, out=img)
    torch.cuda.synchronize()
    print(json.dumps({"case": "fdk_512x512x64_from_512x384x180", "storage": args.storage, **plan.info(),
                      "mean_abs": float(img.abs().mean())}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline / FP64 accuracy leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-FDK measurement")
    ap.add_argument("--no-2d", action="store_true", help="skip the 2D / learned-filter measurements")
    ap.add_argument("--case", choices=["fdk-180v", "fdk-batch", "dd-fan-888x90", "fbp-2d", "lf-train", "lf-apply",
                                        "sf-fan-888x90"],
                    help="run a profiling case instead")
    ap.add_argument("--storage", default="f32", choices=["f32", "bf16", "f16"], help="storage form for --case")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
