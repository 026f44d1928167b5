#!/usr/bin/env python3
"""Throughput and window latency of the supervoxel JFA+Lloyd path on GB300
(one JSON line).

Default workload (stream_720p): the 1280x720 streaming video, 900 frames in
windows of 30 with 10 overlap, 2000 new seeds per window, 20 Lloyd
iterations, on one resident streaming context.
step      one window (asv_stream_push): its new frames up, seed placement,
          metric, LAB, the Lloyd loop (every JFA pass, centroid sums,
          reseeding), post-processing, video-wide labels down.
value     Mvoxel-iterations/s = window voxels x 20 / device time of the
          window's compute (CUDA events; its new frames already in HBM).
e2e       the same metric over asv_stream_push's wall time with pinned host
          buffers; latency_ms p50/p99 of the same calls.
--impl reference
          the CPU restatement of the reference's path (its own GLSL/OpenGL
          pipeline cannot run here) on all host cores, over a 256x144 crop of
          the same video with the same seed spacing, timed over the same
          region (whole windows).  That process loads no library of the GPU
          path (its inputs come from the generator compiled on its own).
Other workloads (--workload): single clips, the 16-clip batch, serving,
connectivity, the whole pipeline, evaluation.
Multi-GPU: replicas only (each rank runs its own stream or clip, no
collective on the data path); value = all ranks' voxel-iterations / max
rank time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("Mvoxel-iterations/s (JFA+Lloyd) and p50/p99 window latency vs plain form at "
          "≥99.9% agreement")
UNIT = "Mvoxel-iterations/s"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC = os.path.join(ROOT, "profiles", "k_jfa_320x240x85.md")
TRAFFIC_720P = os.path.join(ROOT, "profiles", "k_jfa_1280x720x30.md")
# algorithmic bytes per voxel of one JFA pass: label in 4 + label out 4 + LAB 3
JFA_BYTES_PER_VOXEL = 11


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="stream_720p",
                    choices=["clip_320x240x85", "clip_240x160x30", "batch16", "stream_720p",
                             "serve_mix", "connect_320x240x85", "pipeline_320x240x85",
                             "pipeline_png_320x240x85", "quality_320x240x85", "stream_720p_flow"])
    ap.add_argument("--requests", type=int, default=160, help="serve_mix: requests in the run")
    ap.add_argument("--rate", type=float, default=40.0, help="serve_mix: mean arrivals per second")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="stream_720p: skip the per-clip extra key")
    return ap.parse_args()


def workload(name):
    from anisotropic_supervoxel_gb300 import workloads
    return {"clip_320x240x85": workloads.CLIP_320x240x85,
            "clip_240x160x30": workloads.CLIP_240x160x30}[name]


def replicas_value(units_per_rank, seconds, device=None):
    """Whole-job throughput of independent replicas: every rank processed
    `units_per_rank`; the job took the slowest rank's time (max over ranks).
    Returns (units of all ranks / max seconds, max seconds)."""
    import torch
    ws = torch.distributed.get_world_size() if torch.distributed.is_initialized() else 1
    if ws > 1:
        t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        seconds = float(t.item())
    return units_per_rank * ws / seconds, seconds


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi samples (every 50 ms) during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.06)                 # the last sample of the timed region
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 7:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        with open(PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_value(key, path=None):
    """A `key: value` line of a committed k_jfa ncu summary."""
    try:
        with open(path or TRAFFIC) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return float(line.split(":")[1])
    except OSError:
        pass
    return None


def fp32_rate(ops_per_voxel, nvox, launch_s):
    """Executed FP32 operations of a k_jfa pass: ncu's FADD/FMUL counts per
    voxel (two-wide instructions counted twice; the mean of the captured
    steps 3, 2 and 1 in the committed summary) x voxels / the measured
    average pass time."""
    if ops_per_voxel is None or not launch_s:
        return None
    return {"ops_per_voxel_ncu": ops_per_voxel, "tops": ops_per_voxel * nvox / launch_s / 1e12,
            "what": "executed FP32 operations (ncu sass counts, no FMA executes) per voxel of the "
                    "captured passes x voxels / average gather-pass time"}


def jfa_traffic_per_voxel():
    """DRAM bytes per voxel of one JFA pass from the committed ncu summary."""
    return profile_value("dram_bytes_per_voxel")


def cpu_baseline(w, rgb, fwd, bwd, iters):
    from oracle import oracle
    n = os.cpu_count() or 1
    t = time.perf_counter()
    oracle.run_clip(rgb, fwd, bwd, w["K"], iters=iters, nthreads=n, full_ladder=w.get("full_ladder", 0))
    dt = time.perf_counter() - t
    vox = rgb.shape[0] * rgb.shape[1] * rgb.shape[2]
    return {"value": vox * iters / dt / 1e6, "unit": UNIT, "cores": n, "kind": "port",
            "sample": f"{rgb.shape[2]}x{rgb.shape[1]}x{rgb.shape[0]} clip, K={w['K']}, "
                      f"{iters} Lloyd iterations (whole run incl. seed placement and LAB), "
                      f"OpenMP over {n} threads, {dt:.1f} s"}


def config_of(w, name, N):
    return {"workload": f"{name}_K{w['K']}_I{w['iters']}", "W": w["W"], "H": w["H"], "D": w["D"],
            "K": w["K"], "lloyd_iters": w["iters"], "ellipses": w["n_ellipses"],
            "noise_sigma": w["noise_sigma"], "jitter": w["jitter"],
            "jfa_ladder": "full (log2 of the largest dimension)" if w.get("full_ladder") else "reference",
            "variant": "plain", "parallelism": f"replicas{N}",
            "l2": "flushed before every step (512 MiB write)"}


def run_reference(args):
    ws, rank, _ = dist()
    if rank != 0:
        return
    if args.workload == "stream_720p":
        return run_stream_reference(args)
    if args.workload not in ("clip_320x240x85", "clip_240x160x30"):
        print(json.dumps({"impl": "reference", "unavailable": "the CPU arm covers the single-clip "
                          "workloads; " + args.workload + " has no CPU counterpart"}), flush=True)
        return
    w = workload(args.workload)
    from anisotropic_supervoxel_gb300 import workloads
    from oracle import oracle
    rgb, fwd, bwd = workloads.make_clip(w, gen=oracle.synth_clip)
    iters = w["iters"]
    for _ in range(args.warmup):
        cpu_baseline(w, rgb, fwd, bwd, iters)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(w, rgb, fwd, bwd, iters))
    wall = time.perf_counter() - t0
    v = statistics.mean(x["value"] for x in vals)
    cb = dict(vals[-1])
    cb["value"] = v
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipse video, exact generating flow)",
        "config": config_of(w, args.workload, args.gpus),
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own pipeline is GLSL over OpenGL (no graphics stack here); "
                "this arm runs the C restatement of its shader maths and Image.cpp host logic",
    }), flush=True)


def run_ours(args):
    import numpy as np
    import torch

    import anisotropic_supervoxel_gb300 as asv
    from anisotropic_supervoxel_gb300 import workloads

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    if ws > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = workload(args.workload)
    I, K = w["iters"], w["K"]
    rgb, fwd, bwd = workloads.make_clip(w)
    D, H, W, _ = rgb.shape
    nvox = W * H * D

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # --- device-resident value ----------------------------------------------
    full = w.get("full_ladder", 0)
    img = asv.Image(lloyd_iters=I, device=local, full_ladder=full)
    img.init_gpu(rgb, K)
    img.upload_flow(fwd, bwd)
    img.initialization()
    img.seed_matrix()
    img.RGB2LAB()
    img.synchronize()
    st = torch.cuda.ExternalStream(img.stream(), device=torch.device("cuda", local))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    for _ in range(args.warmup):
        img.run_lloyd()
    img.synchronize()
    launches = img.stats().launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = Clocks(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    for k in range(args.steps):
        with torch.cuda.stream(st):
            flush.fill_(k & 255)
        ev[k][0].record(st)
        img.run_lloyd()
        ev[k][1].record(st)
    st.synchronize()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    value, tot_s = replicas_value(nvox * I * args.steps / 1e6, sum(step_ms) / 1e3, f"cuda:{local}")
    tot_ms = tot_s * 1e3
    info = img.info()

    # --- JFA kernel: per-launch device time (CUDA events around each pass) ----
    prof = asv.Image(lloyd_iters=I, device=local, instrument=1, use_graph=0, full_ladder=full)
    prof.init_gpu(rgb, K)
    prof.upload_flow(fwd, bwd)
    prof.initialization()
    prof.seed_matrix()
    prof.RGB2LAB()
    prof.run_lloyd()
    jfa_ms, jfa_n, loop_ms = 0.0, 0, 0.0
    for _ in range(max(1, args.steps)):
        prof.run_lloyd()
        s = prof.stats()
        jfa_ms += s.jfa_ms
        jfa_n += s.jfa_launches
        loop_ms += s.total_ms
    prof.close()
    jfa_launch_s = jfa_ms / jfa_n / 1e3
    peak, peak_kind = peaks()
    achieved = JFA_BYTES_PER_VOXEL * nvox / jfa_launch_s / 1e9
    tpv = jfa_traffic_per_voxel()

    # --- end to end through the C ABI with pinned host buffers ----------------
    def pinned(a):
        t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()

    prgb, pfwd, pbwd = pinned(rgb), pinned(fwd), pinned(bwd)
    plab = torch.empty((D, H, W), dtype=torch.int32, pin_memory=True).numpy()
    e2e = asv.Image(lloyd_iters=I, device=local, full_ladder=full)

    def e2e_step():
        e2e.init_gpu(prgb, K)
        e2e.upload_flow(pfwd, pbwd)
        e2e.initialization()
        e2e.seed_matrix()
        e2e.RGB2LAB()
        e2e.run_lloyd()
        e2e.lib.asv_get_labels(e2e.h, plab.ctypes.data)

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    e2e_val, e2e_s = replicas_value(nvox * I * args.steps / 1e6, time.perf_counter() - t0, f"cuda:{local}")
    ok_labels = bool((plab == img.labels()).all())
    e2e.close()

    # --- centroid sums of the last iteration against an FP64 recomputation ----
    sums = img.sums()
    raw = img.raw_labels().ravel()
    slot = np.where(raw < 0, info.Kp, raw)
    zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    lab4 = img.lab().reshape(-1, 4).astype(np.float64)
    cols = [2.0 * xx.ravel() + 1, 2.0 * yy.ravel() + 1, 2.0 * zz.ravel() + 1, np.ones(nvox),
            lab4[:, 0], lab4[:, 1], lab4[:, 2]]
    ref64 = np.stack([np.bincount(slot, weights=c, minlength=info.Kp + 1) for c in cols], 1)
    sum_err = float(np.max(np.abs(ref64 - sums.astype(np.float64)) / np.maximum(np.abs(ref64), 1.0)))

    cb = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(w, rgb, fwd, bwd, 5)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded ellipse video, exact generating flow)",
            "config": config_of(w, args.workload, ws),
            "e2e": {"value": e2e_val, "unit": UNIT,
                    "h2d_bytes_per_step": int(rgb.nbytes + fwd.nbytes + bwd.nbytes),
                    "d2h_bytes_per_step": int(plab.nbytes),
                    "labels_match_device_run": ok_labels},
            "centroid_sums": {"accumulation": "exact 64-bit integers (fixed point), order-independent",
                              "max_rel_error_vs_fp64": sum_err, "labels": int(info.Kp + 1)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "kernel": "k_jfa", "bytes_per_launch": JFA_BYTES_PER_VOXEL * nvox,
                         "launch_ms": jfa_launch_s * 1e3,
                         "traffic": tpv * nvox if tpv is not None else None,
                         "issue_active_ncu": profile_value("issue_active"),
                         "fp32": fp32_rate(profile_value("fp32_ops_per_voxel"), nvox, jfa_launch_s),
                         "jfa_share_of_loop": jfa_ms / loop_ms if loop_ms else None},
            "clocks": clk,
            "gpu_launches": int(launches * args.steps),
            "kp": info.Kp, "jfa_passes_per_iteration": info.passes,
        }
        if cb is not None:
            line["cpu_baseline"] = cb
        print(json.dumps(line), flush=True)
    img.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def _pct(v, q):
    v = sorted(v)
    if not v:
        return None
    k = min(len(v) - 1, max(0, int(round(q / 100.0 * (len(v) - 1)))))
    return v[k]


def _pinned(a):
    import torch
    t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
    t.numpy()[...] = a
    return t.numpy()


def _line(args, value, ms_per_step, config, extra):
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded ellipse video, exact generating flow)", "config": config}
    line.update(extra)
    print(json.dumps(line), flush=True)


def run_batch16(args):
    """16 clips of uneven size in one context (asv_batch_*): every stage one
    launch over all clips, the Lloyd loop one graph.  Compared with the plain
    per-clip form (one Image per clip, each its own graph) on the same clips."""
    import numpy as np
    import torch

    import anisotropic_supervoxel_gb300 as asv
    from anisotropic_supervoxel_gb300 import workloads
    torch.cuda.set_device(0)
    ws = workloads.batch_clips()
    dims = [(w["W"], w["H"], w["D"], w["K"]) for w in ws]
    clips = [workloads.make_clip(w) for w in ws]
    I = ws[0]["iters"]
    vox_it = sum(W * H * D for W, H, D, _ in dims) * I
    b = asv.Batch(dims, lloyd_iters=I)
    for i, c in enumerate(clips):
        b.upload(i, *c)
    b.prepare()
    zrun = b.autotune()                 # tile depth measured on this batch (asv_autotune)
    b.synchronize()
    st = torch.cuda.ExternalStream(b.stream(), device=torch.device("cuda", 0))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda:0")
    for _ in range(args.warmup):
        b.run_lloyd()
    b.synchronize()
    launches = b.stats().launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = Clocks(0)
    torch.cuda.synchronize()
    clocks.start()
    for k in range(args.steps):
        with torch.cuda.stream(st):
            flush.fill_(k & 255)
        ev[k][0].record(st)
        b.run_lloyd()
        ev[k][1].record(st)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = [x.elapsed_time(y) for x, y in ev]
    value = vox_it * args.steps / (sum(ms) / 1e3) / 1e6
    batch_labels = [b.clip_labels(i) for i in range(len(dims))]

    # plain per-clip form: each clip its own context and graph, run one after another
    imgs = []
    for (W, H, D, K), c in zip(dims, clips):
        im = asv.Image(lloyd_iters=I)
        im.init_gpu(c[0], K)
        im.upload_flow(c[1], c[2])
        im.initialization()
        im.seed_matrix()
        im.RGB2LAB()
        im.run_lloyd()
        imgs.append(im)
    torch.cuda.synchronize()
    same = all(np.array_equal(im.labels(), bl) for im, bl in zip(imgs, batch_labels))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for im in imgs:            # one clip at a time, as the per-clip form runs
            im.run_lloyd()
            im.synchronize()
    plain_s = time.perf_counter() - t0
    plain = vox_it * args.steps / plain_s / 1e6
    for im in imgs:
        im.close()

    # e2e: pinned host clips in, labels out, through the batch API
    pin = [tuple(_pinned(a) for a in c) for c in clips]
    outs = [_pinned(np.empty((D, H, W), np.int32)) for W, H, D, _ in dims]
    lib = b.lib
    for _ in range(2):
        for i, c in enumerate(pin):
            b.upload(i, *c)
        b.prepare()
        b.run_lloyd()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for i, c in enumerate(pin):
            b.upload(i, *c)
        b.prepare()
        b.run_lloyd()
        for i, o in enumerate(outs):
            lib.asv_batch_get_labels(b.h, i, o.ctypes.data)
    e2e_s = time.perf_counter() - t0
    h2d = sum(a.nbytes for c in clips for a in c)
    d2h = sum(o.nbytes for o in outs)
    b.close()
    _line(args, value, sum(ms) / len(ms),
          {"workload": "batch16_uneven", "clips": len(dims),
           "voxels": sum(W * H * D for W, H, D, _ in dims), "K_total": sum(d[3] for d in dims),
           "lloyd_iters": I, "variant": "plain", "parallelism": "replicas1",
           "jfa_zrun": zrun, "tiles": "autotuned (asv_autotune over depths 4/8/16/32)",
           "l2": "flushed before every step (512 MiB write)"},
          {"e2e": {"value": vox_it * args.steps / e2e_s / 1e6, "unit": UNIT,
                   "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
           "plain_per_clip": {"value": plain, "unit": UNIT,
                              "note": "same clips, one context and graph per clip, sequential"},
           "batch_over_plain": value / plain, "labels_equal_plain": same,
           "clocks": clk, "gpu_launches": int(launches * args.steps)})


# crop of the 1280x720 stream timed by the CPU arms and used for the
# agreement check: the 256x144 region at (512, 288) of every frame (1/25 of
# the area) with 1/25 of the new seeds per window: the same voxels per seed,
# so the same seed spacing s = 23 and JFA ladder as the full frame
STREAM_CROP = (512, 288, 256, 144)
STREAM_CROP_SEEDS100 = 10000 // 25


def _stream_windows_frames(n_windows):
    """frames of a video of n_windows stream windows (30 + 20 per further window)"""
    return 30 + 20 * (n_windows - 1)


def _oracle_stream(w, n_windows, nthreads, gen):
    """the oracle's streaming run over the crop video of n_windows windows:
    (labels, blocks, seconds, voxel-iterations)"""
    from anisotropic_supervoxel_gb300 import workloads
    from oracle import oracle
    D_all = _stream_windows_frames(n_windows)
    rgb, fwd, bwd = workloads.stream_frames(w, 0, D_all, gen=gen, crop=STREAM_CROP)
    t = time.perf_counter()
    labels, info = oracle.run_stream(rgb, fwd, bwd, seeds_num_100=STREAM_CROP_SEEDS100, iters=w["iters"],
                                     block_size=w["block_size"], nthreads=nthreads)
    dt = time.perf_counter() - t
    cw, ch = STREAM_CROP[2], STREAM_CROP[3]
    return labels, info["blocks"], dt, info["blocks"] * cw * ch * w["block_size"] * w["iters"], (rgb, fwd, bwd)


def _stream_config(w, ws, device_flow=False):
    return {"workload": "stream_1280x720x900_w30o10_K2000_I20" + ("_device_flow" if device_flow else ""),
            "W": w["W"], "H": w["H"], "frames": w["D_all"], "window": w["block_size"], "overlap": 10,
            "K_window": w["K_window"], "seeds_num_100": w["seeds_num_100"], "lloyd_iters": w["iters"],
            "ellipses": w["n_ellipses"], "noise_sigma": w["noise_sigma"], "variant": "stream",
            "step": "one window: its 20 new frames up, seeds, metric, LAB, 20 Lloyd iterations, "
                    "post-processing, video-wide labels down",
            "parallelism": f"replicas{ws}", "l2": "inputs larger than L2 (each window 27.6 M voxels, ~1.1 GB)"}


def run_stream_720p(args, device_flow=False):
    """The headline: the 1280x720 streaming video (900 frames, windows of 30
    with 10 overlap, 2000 new seeds per window, 20 Lloyd iterations) on one
    resident streaming context.  A step is one window: asv_stream_feed of the
    next window's new frames (a host->device copy on the context's copy
    stream that runs while this window computes), then asv_stream_push_fed of
    this window.  value: window voxel-iterations / device time of the
    window's compute (CUDA events from its first kernel, its new frames
    already in HBM, to its labels mapped); e2e and latency: wall time of the
    step with pinned host buffers (the next window's frames up, compute,
    finished labels down)."""
    import numpy as np
    import torch

    import anisotropic_supervoxel_gb300 as asv
    from anisotropic_supervoxel_gb300 import workloads

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    if ws > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    w = workloads.STREAM_720P
    W, H, D_all, bs, I = w["W"], w["H"], w["D_all"], w["block_size"], w["iters"]
    s100 = w["seeds_num_100"]
    # two pinned sets of new frames: block b is fed from set b % 2 while the
    # block before it computes; a set is refilled only after its block's
    # push has returned
    pins = [{k: _pinned(np.zeros((bs,) + sh, dt)) for k, sh, dt in
             (("rgb", (H, W, 3), np.uint8), ("fwd", (H, W, 2), np.float32), ("bwd", (H, W, 2), np.float32))}
            for _ in range(2)]
    lab_pin = _pinned(np.zeros((bs + bs // 3, H, W), np.int32))   # the longest block (the video's last)

    def new_stream():
        return asv.Stream(W, H, D_all, seeds_num_100=s100, block_size=bs, lloyd_iters=I, device=local)

    def fill(st, b):
        """block b's new frames into pinned set b % 2 (outside the timed region)"""
        _, e, n = st.block(b)
        p = pins[b % 2]
        for key, arr in zip(("rgb", "fwd", "bwd"), workloads.stream_frames(w, e - n, n)):
            p[key][:n] = arr
        return (p["rgb"][:n],) if device_flow else (p["rgb"][:n], p["fwd"][:n], p["bwd"][:n])

    st = new_stream()
    st.feed(*fill(st, 0))
    lat, dev_ms, vox_it, kps, launches, h2d, d2h = [], [], 0, [], 0, 0, 0
    clocks = Clocks(local)
    t_region = 0.0
    for k in range(args.warmup + args.steps):
        if st.info().next_block >= st.info().blocks:        # the video is done: start it again
            st.close()
            st = new_stream()
            st.feed(*fill(st, 0))
        inf = st.info()
        b = inf.next_block
        ahead = fill(st, b + 1) if b + 1 < inf.blocks else None
        if k == args.warmup:
            barrier()
            torch.cuda.synchronize()
            clocks.start()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if ahead is not None:
            st.feed(*ahead)                                  # the next block's upload, during this one
        f0, lab = st.push_fed(out=lab_pin)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            s = st.stats()
            lat.append(dt * 1e3)
            dev_ms.append(s.window_ms)
            launches += s.launches
            vox_it += W * H * (inf.block_end - inf.block_start) * I
            kps.append(st.info().block_Kp)
            h2d += (ahead[0].shape[0] if ahead is not None else 0) * W * H * (3 if device_flow else 19)
            d2h += lab.nbytes
            t_region += dt
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    st.close()
    value, dev_s = replicas_value(vox_it / 1e6, sum(dev_ms) / 1e3, f"cuda:{local}")
    e2e_sync, _ = replicas_value(vox_it / 1e6, t_region, f"cuda:{local}")

    # e2e, pipelined: the same video from its start on a new streaming
    # context; every timed step copies its window's new frames into a pinned
    # set, feeds them (copy stream), enqueues the window
    # (asv_stream_push_fed_async) and waits for the window before it
    # (asv_stream_wait: its labels in host memory), so the host's work for
    # one window overlaps the device's work on the other.  The frames are
    # generated before the timed region (generation takes longer than a
    # window).  K_e2e windows, at most 12 (5 GB of frames held).
    k_e2e = min(args.steps, 12)
    w2 = 2                                                 # warm-up windows of this phase
    st2 = new_stream()
    pre = []
    for b in range(w2 + k_e2e + 1):
        _, e, n = st2.block(b)
        pre.append(workloads.stream_frames(w, e - n, n))
    labs = [_pinned(np.zeros((bs + bs // 3, H, W), np.int32)) for _ in range(2)]

    def put(b):
        """window b's frames into pinned set b % 2"""
        n = pre[b][0].shape[0]
        p = pins[b % 2]
        for key, arr in zip(("rgb", "fwd", "bwd"), pre[b]):
            p[key][:n] = arr
        return (p["rgb"][:n],) if device_flow else (p["rgb"][:n], p["fwd"][:n], p["bwd"][:n])

    st2.feed(*put(0))
    for b in range(w2):
        st2.feed(*put(b + 1))
        st2.push_fed(out=labs[b % 2])
    torch.cuda.synchronize()
    barrier()
    t_p0 = time.perf_counter()
    st2.push_fed_async(labs[w2 % 2])
    vox_p = 0
    for j in range(k_e2e):
        b = w2 + j
        if j + 1 < k_e2e:
            st2.feed(*put(b + 1))                           # set (b+1) % 2: its window b-1 has finished
            st2.push_fed_async(labs[(b + 1) % 2])
        f0, lab = st2.wait()
        blk = st2.block(b)
        vox_p += W * H * (blk[1] - blk[0]) * I
    torch.cuda.synchronize()
    barrier()
    t_p = time.perf_counter() - t_p0
    st2.close()
    del pre
    e2e_val, e2e_s = replicas_value(vox_p / 1e6, t_p, f"cuda:{local}")

    # k_jfa per launch at this size: the Lloyd loop of the video's first 30
    # frames (2000 seeds, stream variant) with a CUDA event around every pass
    rgb, fwd, bwd = workloads.stream_frames(w, 0, bs)
    prof = asv.Image(lloyd_iters=I, device=local, instrument=1, use_graph=0, variant=1)
    prof.init_gpu(rgb, w["K_window"])
    prof.upload_flow(fwd, bwd)
    prof.initialization()
    prof.seed_matrix()
    prof.RGB2LAB()
    prof.run_lloyd()
    jfa_ms, jfa_n, loop_ms = 0.0, 0, 0.0
    for _ in range(3):
        prof.run_lloyd()
        s = prof.stats()
        jfa_ms += s.jfa_ms
        jfa_n += s.jfa_launches
        loop_ms += s.total_ms
    prof.close()
    nvox = W * H * bs
    jfa_launch_s = jfa_ms / jfa_n / 1e3
    peak, peak_kind = peaks()
    achieved = JFA_BYTES_PER_VOXEL * nvox / jfa_launch_s / 1e9
    tpv = profile_value("dram_bytes_per_voxel", TRAFFIC_720P)

    # agreement with the oracle on the crop sample (the same windows the CPU
    # arm times), and the CPU baseline itself
    cb = agree = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        n_win = 2
        want, nb, cpu_s, cpu_vox, (crgb, cfwd, cbwd) = _oracle_stream(w, n_win, os.cpu_count() or 1, None)
        cw, ch = STREAM_CROP[2], STREAM_CROP[3]
        cst = asv.Stream(cw, ch, crgb.shape[0], seeds_num_100=STREAM_CROP_SEEDS100, block_size=bs, lloyd_iters=I,
                         device=local)
        got = np.full(want.shape, -7, np.int32)
        for _ in range(cst.info().blocks):
            ci = cst.info()
            a0 = ci.block_end - ci.frames_needed
            f0, lab = cst.push(crgb[a0:ci.block_end], cfwd[a0:ci.block_end], cbwd[a0:ci.block_end])
            got[f0:f0 + lab.shape[0]] = lab
        cst.close()
        agree = {"voxels": int(want.size), "equal": float((got == want).mean()), "bit_exact": bool((got == want).all()),
                 "sample": f"{cw}x{ch} crop at ({STREAM_CROP[0]}, {STREAM_CROP[1]}) of frames 0-{want.shape[0] - 1}, "
                           f"{nb} windows, {I} iterations, seeds_num_100 {STREAM_CROP_SEEDS100} (same seed spacing)",
                 "against": "the oracle (CPU restatement of the reference's shaders and Render/Image host logic)"}
        cb = {"value": cpu_vox / cpu_s / 1e6, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
              "sample": f"the oracle's streaming run over a {cw}x{ch} crop of the same video (frames 0-"
                        f"{want.shape[0] - 1}, {nb} windows of 30, 20 iterations, 1/25 of the seeds: the same seed "
                        f"spacing and JFA ladder), OpenMP over {os.cpu_count()} threads, {cpu_s:.1f} s"}

    extra = {}
    if rank == 0 and ws == 1 and not getattr(args, "no_extras", False):
        extra["clip_320x240x85"] = _clip_rate(args, workloads.CLIP_320x240x85, local)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded ellipse video with background drift, exact generating flow"
                    + ("; flow computed on the device" if device_flow else "") + ")",
            "config": _stream_config(w, ws, device_flow),
            "latency_ms": {"p50": _pct(lat, 50), "p99": _pct(lat, 99), "max": max(lat), "windows": len(lat),
                           "device_p50": _pct(dev_ms, 50), "device_p99": _pct(dev_ms, 99),
                           "what": "wall time per window of asv_stream_feed (the next window's frames, "
                                   "uploaded on a copy stream during this one) + asv_stream_push_fed (this "
                                   "window's compute, its labels down into a pinned buffer); device_*: its "
                                   "compute alone", "target_p99": 33.0},
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
                    "d2h_bytes_per_step": int(d2h / args.steps), "windows": k_e2e,
                    "what": "pipelined windows through asv_stream_feed + asv_stream_push_fed_async + "
                            "asv_stream_wait (per window: new frames copied into pinned memory and up, "
                            "compute, labels down), wall time of the whole run",
                    "sync": e2e_sync},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "kernel": "k_jfa",
                         "bytes_per_launch": JFA_BYTES_PER_VOXEL * nvox, "launch_ms": jfa_launch_s * 1e3,
                         "launch_of": "a k_jfa gather pass over one 1280x720x30 window (27.6 M voxels)",
                         "traffic": tpv * nvox if tpv is not None else None,
                         "issue_active_ncu": profile_value("issue_active", TRAFFIC_720P),
                         "fp32": fp32_rate(profile_value("fp32_ops_per_voxel", TRAFFIC_720P), nvox, jfa_launch_s),
                         "jfa_share_of_loop": jfa_ms / loop_ms if loop_ms else None},
            "block_Kp_mean": statistics.mean(kps),
            "clocks": clk, "gpu_launches": int(launches),
        }
        if agree is not None:
            line["agreement"] = agree
        if cb is not None:
            line["cpu_baseline"] = cb
        line.update(extra)
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def _clip_rate(args, w, local, steps=5):
    """the per-clip form on one clip (extra key of the headline line):
    device-timed Lloyd loop with inputs resident, and end to end"""
    import torch

    import anisotropic_supervoxel_gb300 as asv
    from anisotropic_supervoxel_gb300 import workloads
    rgb, fwd, bwd = workloads.make_clip(w)
    D, H, W, _ = rgb.shape
    img = asv.Image(lloyd_iters=w["iters"], device=local)
    img.init_gpu(rgb, w["K"])
    img.upload_flow(fwd, bwd)
    img.initialization()
    img.seed_matrix()
    img.RGB2LAB()
    for _ in range(3):
        img.run_lloyd()
    img.synchronize()
    st = torch.cuda.ExternalStream(img.stream(), device=torch.device("cuda", local))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    ms = []
    for k in range(steps):
        with torch.cuda.stream(st):
            flush.fill_(k & 255)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        img.run_lloyd()
        e1.record(st)
        st.synchronize()
        ms.append(e0.elapsed_time(e1))
    img.close()
    vox_it = W * H * D * w["iters"]
    return {"value": vox_it / (sum(ms) / len(ms) / 1e3) / 1e6, "unit": UNIT, "ms_per_loop": sum(ms) / len(ms),
            "workload": f"clip_{W}x{H}x{D}_K{w['K']}_I{w['iters']}, Lloyd loop on the device, inputs resident"}


def run_stream_reference(args):
    """The CPU arm of the headline: the oracle's streaming run (the
    reference's path restated on the host cores) over the 256x144 crop of the
    same video, which keeps the per-voxel work (seed spacing, JFA ladder).
    W untimed warm-up windows, then a video of exactly K windows timed.  Its
    inputs come from the generator compiled on its own (oracle.synth_clip):
    this process loads no library of the GPU path."""
    ws, rank, _ = dist()
    if rank != 0:
        return
    from anisotropic_supervoxel_gb300 import workloads
    from oracle import oracle
    w = workloads.STREAM_720P
    n = os.cpu_count() or 1
    if args.warmup > 0:
        _oracle_stream(w, args.warmup, n, oracle.synth_clip)
    labels, nb, dt, vox, _ = _oracle_stream(w, args.steps, n, oracle.synth_clip)
    v = vox / dt / 1e6
    cw, ch = STREAM_CROP[2], STREAM_CROP[3]
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipse video with background drift, exact generating flow)",
        "config": _stream_config(w, 1),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": n, "kind": "port",
                         "sample": f"{cw}x{ch} crop at ({STREAM_CROP[0]}, {STREAM_CROP[1]}) of the video, {nb} windows "
                                   f"of 30 frames (the first {nb}), 20 iterations, 1/25 of the seeds (the same seed "
                                   f"spacing and JFA ladder as the full frame); OpenMP over {n} threads; {dt:.1f} s"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "windows_timed": nb,
        "note": "the reference's own pipeline is GLSL over OpenGL (no graphics stack here); this arm runs the "
                "C restatement of its shader maths and Render/Image host logic, timed over the same region "
                "as the GPU arm (a whole window: seeds, metric, LAB, the Lloyd loop, post-processing)",
    }), flush=True)


def run_serve_mix(args):
    """Poisson arrivals of mixed requests through the request pool
    (asv_server_*): 50% 240x160x30 K=200 clips, 35% 640x480x60 K=1000 clips,
    15% 720p 30-frame streaming windows K=2000 (two sessions), 120 GB HBM
    budget.  Latency = submit -> labels on the host."""
    import numpy as np
    import torch

    import anisotropic_supervoxel_gb300 as asv
    from anisotropic_supervoxel_gb300 import workloads
    torch.cuda.set_device(0)
    rng = np.random.default_rng(20240605)
    mix = workloads.serving_mix()
    n = args.requests
    kinds = rng.choice(len(mix), size=n, p=[m[0] for m in mix])
    gaps = rng.exponential(1.0 / args.rate, size=n)
    # input pools (two clips per clip class, reused; one 30- and one 20-frame window)
    pools = {}
    for c in (0, 1):
        w = dict(mix[c][1])
        pools[c] = []
        for j in range(2):
            w["seed"] = 777 + 10 * c + j
            pools[c].append(tuple(_pinned(a) for a in workloads.make_clip(w)))
    ww = mix[2][1]
    win = {}
    for nf, f0 in ((30, 0), (20, 30)):
        win[nf] = tuple(_pinned(a) for a in asv.synth_clip(
            ww["W"], ww["H"], nf, n_ellipses=ww["n_ellipses"], noise_sigma=ww["noise_sigma"],
            vmax=ww["vmax"], seed=4242, frame0=f0))
    n_sess = 2
    per_sess = [0] * n_sess
    plan = []
    for i, k in enumerate(kinds):
        if k == 2:
            s = sum(per_sess) % n_sess
            plan.append((2, s, per_sess[s]))
            per_sess[s] += 1
        else:
            plan.append((int(k), i % 2, 0))
    budget = 120 << 30
    srv = asv.Server(max_slots=6, hbm_budget=budget, lloyd_iters=10)
    sids = []
    for s in range(n_sess):
        nw = max(per_sess[s], 1)
        sids.append(srv.open_session(ww["W"], ww["H"], 30 + 20 * (nw - 1),
                                     seeds_num_100=ww["K"] * 100 // 20))
    # warm-up: one request of each clip class
    for c in (0, 1):
        srv.wait(srv.submit_clip(*pools[c][0], mix[c][1]["K"]))
    clocks = Clocks(0)
    clocks.start()
    ids, vox = [], 0
    t0 = time.perf_counter()
    t_next = t0
    for (k, j, b), g in zip(plan, gaps):
        t_next += g
        now = time.perf_counter()
        if t_next > now:
            time.sleep(t_next - now)
        if k == 2:
            nf = 30 if b == 0 else 20
            ids.append((k, srv.submit_window(sids[j], *win[nf])))
            vox += ww["W"] * ww["H"] * 30 * 10
        else:
            w = mix[k][1]
            ids.append((k, srv.submit_clip(*pools[k][j], w["K"])))
            vox += w["W"] * w["H"] * w["D"] * 10
    lat, qd = {0: [], 1: [], 2: []}, {0: [], 1: [], 2: []}
    for k, rid in ids:
        _, ms, qms = srv.wait(rid)
        lat[k].append(ms)
        qd[k].append(qms)
    t_end = time.perf_counter()
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    allv = lat[0] + lat[1] + lat[2]
    span = t_end - t0
    value = vox / span / 1e6
    names = ["clip_240x160x30", "clip_640x480x60", "window_1280x720x30"]
    _line(args, value, span * 1e3 / n,
          {"workload": "serve_poisson_mix", "requests": n, "rate_per_s": args.rate,
           "mix": "50% 240x160x30 K200, 35% 640x480x60 K1000, 15% 720p 30-frame windows K2000",
           "hbm_budget_gb": 120, "slots": 6, "sessions": n_sess, "lloyd_iters": 10,
           "parallelism": "replicas1", "l2": "inputs larger than L2"},
          {"latency_ms": {"p50": _pct(allv, 50), "p99": _pct(allv, 99),
                          **{nm: {"p50": _pct(lat[i], 50), "p99": _pct(lat[i], 99), "n": len(lat[i]),
                                  "queue_p50": _pct(qd[i], 50), "queue_p99": _pct(qd[i], 99)}
                             for i, nm in enumerate(names)}},
           "requests_per_s": n / span, "failed": st.failed,
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": None,
                   "d2h_bytes_per_step": None},
           "clocks": clk})


def run_connect(args):
    """3D connectivity enforcement (Image::enforce_connectivity_3d) on the raw
    labels of the 320x240x85 clip after its Lloyd loop; step = one
    asv_enforce_connectivity on the device labels (labels back to the host
    included).  CPU baseline: the oracle's restatement of the reference's
    sequential scan (pinned to the reference's C++) on the same labels."""
    import numpy as np
    import torch

    import anisotropic_supervoxel_gb300 as asv
    from anisotropic_supervoxel_gb300 import workloads
    torch.cuda.set_device(0)
    w = workloads.CLIP_320x240x85
    rgb, fwd, bwd = workloads.make_clip(w)
    D, H, W, _ = rgb.shape
    n = W * H * D
    img = asv.Image(lloyd_iters=w["iters"])
    img.segment(rgb, fwd, bwd, w["K"])
    raw = img.raw_labels()
    supsz = n // w["K"]
    for _ in range(args.warmup):
        got, num = img.enforce_connectivity()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        got, num = img.enforce_connectivity()
    dt = (time.perf_counter() - t0) / args.steps
    from oracle import oracle
    t1 = time.perf_counter()
    want, m = oracle.enforce_connectivity(raw, supsz)
    cpu_dt = time.perf_counter() - t1
    img.close()
    _line(args, n / dt / 1e6, dt * 1e3,
          {"workload": "connect_320x240x85", "supsz": supsz, "parallelism": "replicas1",
           "l2": "labels (26 MB) and scratch (200 MB) exceed the working set of one pass"},
          {"metric": "Mvoxel/s of 3D connectivity enforcement", "unit": "Mvoxel/s", "dtype": "int32",
           "labels_equal_oracle": bool(np.array_equal(got, want)) and num == m, "label_num": num,
           "cpu_baseline": {"value": n / cpu_dt / 1e6, "unit": "Mvoxel/s", "cores": 1, "kind": "port",
                            "sample": f"the same {W}x{H}x{D} labels, the oracle's sequential scan, "
                                      f"{cpu_dt:.2f} s"},
           "e2e": {"value": n / dt / 1e6, "unit": "Mvoxel/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": int(4 * n)}})


def run_pipeline(args, from_png=False):
    """The whole Render::run on the device for the 320x240x85 clip: raw BGR
    frames (top row first) up from pinned memory, preprocessing
    (asv_init_gpu_bgr), the forward/backward optical flow (asv_compute_flow,
    in place of OpenCV's Farneback), seed placement, metric, LAB, the Lloyd
    loop, labels back.  from_png: the step starts from the 85 frames as PNG
    files (written once, untimed) and decodes them on the host threads
    (asv_png_read_frames_bgr, the imread loop of Render::run).
    value = voxel-iterations / wall time of that step."""
    import numpy as np
    import torch

    import anisotropic_supervoxel_gb300 as asv
    from anisotropic_supervoxel_gb300 import workloads
    torch.cuda.set_device(0)
    w = workloads.CLIP_320x240x85
    rgb, _, _ = workloads.make_clip(w)
    bgr = _pinned(np.ascontiguousarray(rgb[:, ::-1, :, ::-1]))      # as read from a video
    D, H, W, _ = rgb.shape
    n, I, K = W * H * D, w["iters"], w["K"]
    out = _pinned(np.empty((D, H, W), np.int32))
    img = asv.Image(lloyd_iters=I)
    lib = img.lib
    tmp = tempfile.TemporaryDirectory() if from_png else None
    paths, png_bytes, decode_ms = [], 0, []
    if from_png:
        for t in range(D):
            paths.append(os.path.join(tmp.name, f"{t + 1:05d}.png"))
            asv.write_png(paths[-1], bgr[t][..., ::-1])
            png_bytes += os.path.getsize(paths[-1])

    def step(timed):
        ev = None
        if timed:
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        if from_png:
            t0 = time.perf_counter()
            asv.read_frames(paths, out=bgr)
            decode_ms.append((time.perf_counter() - t0) * 1e3)
        img.init_gpu_bgr(bgr, K)
        st = torch.cuda.ExternalStream(img.stream(), device=torch.device("cuda", 0))
        if ev:
            ev[0].record(st)
        img.compute_flow()
        if ev:
            ev[1].record(st)
        img.initialization()
        img.seed_matrix()
        img.RGB2LAB()
        img.run_lloyd()
        lib.asv_get_labels(img.h, out.ctypes.data)
        if ev:
            ev[2].record(st)
        return ev

    for _ in range(args.warmup):
        step(False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    evs = [step(True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / args.steps
    flow_ms = statistics.mean(e[0].elapsed_time(e[1]) for e in evs)
    img.close()
    extra = {"flow_ms": flow_ms, "flow_pairs": 2 * (D - 1),
             "e2e": {"value": n * I / dt / 1e6, "unit": UNIT, "h2d_bytes_per_step": int(bgr.nbytes),
                     "d2h_bytes_per_step": int(out.nbytes)},
             "note": "flow by this library's Farneback implementation (OpenCV's is not available)"}
    if from_png:
        tmp.cleanup()
        extra.update({"png_decode_ms": statistics.median(decode_ms[-args.steps:]), "png_bytes": png_bytes,
                      "decode_threads": os.cpu_count()})
    _line(args, n * I / dt / 1e6, dt * 1e3,
          {"workload": ("pipeline_png" if from_png else "pipeline") + "_320x240x85_K1000_I15",
           "parallelism": "replicas1",
           "l2": "inputs larger than L2 (19.6 MB frames, 80 MB working set, flow scratch 1.1 GB)"},
          extra)


def run_quality(args):
    """LIBSVX-style quality of the 320x240x85 clip's supervoxels against the
    generator's ground truth (asv_evaluate), with the exact generating flow
    and with the device optical flow; value = evaluation throughput."""
    import torch

    import anisotropic_supervoxel_gb300 as asv
    from anisotropic_supervoxel_gb300 import workloads
    torch.cuda.set_device(0)
    w = workloads.CLIP_320x240x85
    rgb, fwd, bwd = workloads.make_clip(w)
    truth = asv.synth_truth(w["W"], w["H"], w["D"], n_ellipses=w["n_ellipses"], noise_sigma=w["noise_sigma"],
                            vmax=w["vmax"], jitter=w["jitter"], seed=w["seed"])
    n = rgb.shape[0] * rgb.shape[1] * rgb.shape[2]
    img = asv.Image(lloyd_iters=w["iters"])
    given = img.segment(rgb, fwd, bwd, w["K"])
    img.init_gpu(rgb, w["K"])
    img.compute_flow()
    img.initialization()
    img.seed_matrix()
    img.RGB2LAB()
    img.run_lloyd()
    computed = img.labels()
    conn, _ = img.enforce_connectivity()
    for _ in range(args.warmup):
        img.evaluate(given, truth)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        q_given = img.evaluate(given, truth)
    dt = (time.perf_counter() - t0) / args.steps
    q_flow = img.evaluate(computed, truth)
    q_conn = img.evaluate(conn, truth)
    img.close()
    _line(args, n / dt / 1e6, dt * 1e3,
          {"workload": "quality_320x240x85_K1000_I15", "parallelism": "replicas1",
           "l2": "labels and truth (52 MB) uploaded every step"},
          {"metric": "Mvoxel/s of supervoxel evaluation (LIBSVX-style measures)", "unit": "Mvoxel/s",
           "dtype": "int32",
           "quality": {"generating_flow": q_given, "device_flow": q_flow,
                       "generating_flow_connectivity_enforced": q_conn},
           "e2e": {"value": n / dt / 1e6, "unit": "Mvoxel/s", "h2d_bytes_per_step": int(8 * n),
                   "d2h_bytes_per_step": 0}})


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch16":
        run_batch16(args)
    elif args.workload == "stream_720p":
        run_stream_720p(args)
    elif args.workload == "stream_720p_flow":
        run_stream_720p(args, device_flow=True)
    elif args.workload == "serve_mix":
        run_serve_mix(args)
    elif args.workload == "connect_320x240x85":
        run_connect(args)
    elif args.workload == "pipeline_320x240x85":
        run_pipeline(args)
    elif args.workload == "pipeline_png_320x240x85":
        run_pipeline(args, from_png=True)
    elif args.workload == "quality_320x240x85":
        run_quality(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
