"""Benchmark of the GB300 descale executor on the Delanczos YUV420P16 workload.

Workload (one "step"): Delanczos(taps=3) of 64 YUV420P16 frames
1920x1080 -> 1440x810 (chroma 960x540 -> 720x405), f64mode=0 (auto: the
plans are well conditioned, so the Float32 route), padding=1 (repeat), the
plugin's chroma placement.  Synthetic frames: per plane a seeded uniform
[0,1] base at the target size, Gaussian blur sigma 1.5, bicubic (b=0,
c=0.5) upscale to the source size, N(0, 1e-3) noise, limited-range 16-bit
quantisation.  The 64 frames (398 MB in, 224 MB out) exceed the 129 MB L2,
so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  `value` is Mpix/s of source pixels summed
over planes with inputs resident in HBM; `e2e` is the same metric through
the synchronous host-frame C-ABI calls (pinned host planes, copies inside
the timed region), beside it the same step as per-plane calls from 16
Python threads and from 16 C++ threads (bench_host_calls.cpp); `roofline` divides the algorithmic bytes of a step (the
sum over its kernel launches, each counted by the executor) by the step's
CUDA-event time: the prepared batch runs as two parts on two streams whose
kernels overlap, so the per-kernel event times (also reported, as shares)
add up to more than the step.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "vapoursynth-descalemvc_gb300"))

SRC_W, SRC_H, DST_W, DST_H = 1920, 1080, 1440, 810
FRAMES = 64
KERNEL = dict(kernel="lanczos", taps=3, b=0.0, c=0.5, blur=1.0, border="repeat", f64_mode=0)
METRIC = "descale Mpix/s (source pixels, Delanczos YUV420P16 1920x1080->1440x810)"
# DRAM bytes (read + write) per frame of both passes: dram__bytes_read.sum +
# dram__bytes_write.sum of the rows and columns pass from one ncu capture of
# a 24-frame cut of this workload, divided by 24 (traffic grows with the
# frame count).
DRAM_BYTES_PER_FRAME = 619.8e6 / 24
TRAFFIC_SOURCE = ("ncu capture (dram__bytes_read.sum + dram__bytes_write.sum, both passes) of a "
                  "24-frame cut of this workload, scaled to the step's frames")


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def max_over_ranks(value, dist, device):
    """The largest `value` over the ranks (the slowest replica's time)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_step, world, steps, elapsed_ms):
    """Units of all replicas per second in millions: every rank processes
    `units_per_step` per step (weak scaling), the job takes the slowest
    rank's time."""
    return world * steps * units_per_step / (elapsed_ms / 1e3) / 1e6


def link_bandwidth(h2d_bytes, d2h_bytes):
    """Host<->device copy bandwidth of pinned buffers of the step's sizes:
    each direction alone and both at once on two streams (the roofline of
    the end-to-end figure)."""
    import torch
    up_h = torch.empty(h2d_bytes, dtype=torch.uint8, pin_memory=True)
    up_d = torch.empty(h2d_bytes, dtype=torch.uint8, device="cuda")
    dn_h = torch.empty(d2h_bytes, dtype=torch.uint8, pin_memory=True)
    dn_d = torch.empty(d2h_bytes, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    def both():
        with torch.cuda.stream(s1):
            up_d.copy_(up_h, non_blocking=True)
        with torch.cuda.stream(s2):
            dn_h.copy_(dn_d, non_blocking=True)

    t_up = timed(lambda: up_d.copy_(up_h, non_blocking=True))
    t_dn = timed(lambda: dn_h.copy_(dn_d, non_blocking=True))
    t_both = timed(both)
    return {"h2d_gbs": h2d_bytes / t_up / 1e9, "d2h_gbs": d2h_bytes / t_dn / 1e9,
            "concurrent_gbs": (h2d_bytes + d2h_bytes) / t_both / 1e9}


def plane_requests(gb):
    """Luma and chroma (4:2:0, left-aligned chroma placement) requests, as
    prepare_filter_requests builds them (src/vs_plugin.cpp:656-705)."""
    cs_w, cs_h = SRC_W >> 1, SRC_H >> 1
    shift = 0.25 - 0.25 * DST_W / SRC_W
    return {
        "luma_h": gb.AxisRequest(SRC_W, DST_W, float(DST_W), 0.0, **KERNEL),
        "luma_v": gb.AxisRequest(SRC_H, DST_H, float(DST_H), 0.0, **KERNEL),
        "chroma_h": gb.AxisRequest(cs_w, DST_W >> 1, DST_W * cs_w / SRC_W, shift, **KERNEL),
        "chroma_v": gb.AxisRequest(cs_h, DST_H >> 1, DST_H * cs_h / SRC_H, 0.0, **KERNEL),
    }


def _upscale_matrix(arrays, src, dst):
    """Forward bicubic (b=0, c=0.5) resampling dst -> src: the descale
    matrix A of a plan, rebuilt from its A^T CSR.  `arrays(src, dst)` returns
    the plan's (transpose_weights, transpose_indices, transpose_offsets)."""
    import scipy.sparse as sp
    w, idx, off = arrays(src, dst)
    at = sp.csr_matrix((np.asarray(w, np.float64), idx, off), shape=(dst, src))
    return at.T.tocsr()


def product_arrays(gb):
    """Upscaler arrays from this executor's planner (the GPU arm)."""
    def arrays(src, dst):
        p = gb.AxisPlan(gb.AxisRequest(src, dst, float(dst), 0.0, "bicubic", 3, 0.0, 0.5, 1.0,
                                       "symmetric", 1), cached=False)
        return (p.array("transpose_weights"), p.array("transpose_indices"),
                p.array("transpose_offsets"))
    return arrays


def checker_arrays(mod, O):
    """Upscaler arrays from the reference engine's planner (or the oracle's,
    which is bit-identical): the CPU arm synthesises its frames without
    loading the executor library."""
    def arrays(src, dst):
        p = mod.Plan(O.make_request(src, dst, float(dst), 0.0, "bicubic", 3, 0.0, 0.5, 1.0,
                                    "symmetric", 1))
        return p.transpose_weights, p.transpose_indices, p.transpose_offsets
    return arrays


def make_frames(arrays, frames, seed):
    """Seeded synthetic YUV420P16 frames (see the module docstring)."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    mats = {}
    out = []
    for _ in range(frames):
        planes = []
        for idx, (sw, sh, dw, dh) in enumerate([(SRC_W, SRC_H, DST_W, DST_H),
                                                 (SRC_W >> 1, SRC_H >> 1, DST_W >> 1, DST_H >> 1),
                                                 (SRC_W >> 1, SRC_H >> 1, DST_W >> 1, DST_H >> 1)]):
            key = (sw, sh, dw, dh)
            if key not in mats:
                mats[key] = (_upscale_matrix(arrays, sw, dw), _upscale_matrix(arrays, sh, dh))
            ah, av = mats[key]
            base = gaussian_filter(rng.random((dh, dw)), 1.5)
            up = av @ (ah @ base.T).T
            up = up + rng.normal(0.0, 1e-3, up.shape)
            if idx == 0:
                q = np.rint(up * 56064.0 + 4096.0)
            else:
                q = np.rint((up - 0.5) * 57344.0 + 32768.0)
            planes.append(np.clip(q, 0, 65535).astype(np.uint16))
        out.append(planes)
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region
    (every 10 ms by default)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device, period_ms=10):
        self.device = device
        self.period_ms = period_ms
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() in ("active", "1"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def pixels_per_frame():
    return SRC_W * SRC_H + 2 * (SRC_W >> 1) * (SRC_H >> 1)


def host_threads():
    """Host threads this process may run on (os.sched_getaffinity), and how
    that was found."""
    try:
        return len(os.sched_getaffinity(0)), "os.sched_getaffinity(0)"
    except (AttributeError, OSError):
        return os.cpu_count() or 1, "os.cpu_count()"


def checker_modules():
    """The oracle and, where it was built on this machine, the reference
    engine (oracle/_ref): (oracle, reference-or-None)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    try:
        import reference as R
        if not R.available():
            R = None
    except Exception:
        R = None
    return O, R


def cpu_baseline(frames, threads, budget_s=12.0, route="automatic"):
    """The reference's own CPU engine (oracle/_ref, built from its sources
    on this machine) on the host cores, whole frames through its 2D integer
    route, one frame per thread; the oracle port of its scalar route where
    the engine is absent.  route: "automatic" (the engine's own pick: NEON
    on aarch64, AVX-512/AVX2 on x86) or "scalar"."""
    O, R = checker_modules()
    mod = R if R is not None else O
    kind = "reference" if R is not None else "port"
    if R is None:
        route = "scalar"
    path = 1 if route == "automatic" else 0
    reqs = {
        "luma_h": (SRC_W, DST_W, float(DST_W), 0.0), "luma_v": (SRC_H, DST_H, float(DST_H), 0.0),
        "chroma_h": (SRC_W >> 1, DST_W >> 1, DST_W * (SRC_W >> 1) / SRC_W, 0.25 - 0.25 * DST_W / SRC_W),
        "chroma_v": (SRC_H >> 1, DST_H >> 1, DST_H * (SRC_H >> 1) / SRC_H, 0.0)}
    plans = {k: mod.Plan(O.make_request(*v, "lanczos", 3, 0.0, 0.5, 1.0, "repeat", 0))
             for k, v in reqs.items()}
    luma = (4096.0, float(np.float32(1) / np.float32(56064)), 56064.0, 4096.0, 65535)
    chroma = (32768.0, float(np.float32(1) / np.float32(57344)), 57344.0, 32768.0, 65535)

    def one(frame):
        y, u, v = frame
        out = []
        for plane, (h, vv, conv) in zip((y, u, v), [("luma_h", "luma_v", luma),
                                                    ("chroma_h", "chroma_v", chroma),
                                                    ("chroma_h", "chroma_v", chroma)]):
            if R is not None:
                out.append(R.inverse_2d(plans[h], plans[vv], plane, conv, path=path))
            else:
                out.append(O.inverse_2d(plans[h], plans[vv], plane, conv))
        return out

    one(frames[0])  # warm-up
    done, t0 = 0, time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as pool:
        while time.perf_counter() - t0 < budget_s or done == 0:
            batch = [frames[(done + i) % len(frames)] for i in range(threads)]
            list(pool.map(one, batch))
            done += len(batch)
    elapsed = time.perf_counter() - t0
    isa = os.uname().machine
    what = (f"reference engine CpuPath::{route} ({'NEON' if isa == 'aarch64' else 'AVX-512/AVX2'} "
            f"route on {isa})" if route == "automatic" else f"reference engine CpuPath::scalar on {isa}") \
        if kind == "reference" else f"oracle port of the scalar route on {isa}"
    return {"value": done * pixels_per_frame() / elapsed / 1e6, "unit": "Mpix/s",
            "cores": threads, "kind": kind, "route": route,
            "sample": f"{done} frames (YUV420P16 1920x1080->1440x810, Delanczos taps=3), "
                      f"{threads} threads x 1 frame, {what}, {elapsed:.1f} s"}


def run_reference(args, rank, world):
    """The reference arm: the reference's own CPU engine (built from its
    sources on this machine into oracle/_ref) on every host thread, through
    its optimized route (CpuPath::automatic), one frame per thread, with the
    scalar route timed beside it; the oracle port of the scalar route where
    the engine could not be built.  The frames are synthesised with the
    reference planner's own upscaler: the executor library is not loaded."""
    if rank != 0:
        return
    O, R = checker_modules()
    frames = make_frames(checker_arrays(R if R is not None else O, O), 4, 1234)
    threads, how = host_threads()
    per_step = max(1.5, 30.0 / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_baseline(frames, threads, budget_s=0.1)
    results = [cpu_baseline(frames, threads, budget_s=per_step) for _ in range(args.steps)]
    value = float(np.mean([r["value"] for r in results]))
    scalar = cpu_baseline(frames, threads, budget_s=4.0, route="scalar") if R is not None else None
    ms = pixels_per_frame() * FRAMES / (value * 1e6) * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mpix/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(),
            "cpu_baseline": dict(results[-1], value=value, cores_source=how),
            "scalar_route": scalar,
            "e2e": {"value": value, "unit": "Mpix/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    if R is None:
        line["note"] = "reference engine not built on this machine: oracle port of the scalar route"
    print(json.dumps(line), flush=True)


SWEEP_W, SWEEP_H = 1920, 1080
SWEEP_HEIGHTS = range(500, 1001)
SWEEP_METRIC = "candidate solves/s (1920x1080 GRAYS sweep, heights 500..1000, 3 kernels)"


def run_sweep(args, rank, world):
    """Batched candidate sweep: one 1920x1080 GRAYS float32 frame built from a
    hidden base height drawn from the seed in [600, 900], descaled to every
    height 500..1000 (width round(16 h / 9), even) with Debicubic(0, 0.5),
    Debilinear and Delanczos(3), each result re-upscaled and scored by mean
    absolute error: 1503 candidates per step, one CUDA graph per step.  Warm
    = plans resident; cold = host planning + sweep preparation + one run;
    plain = the same candidates one at a time, each waited for."""
    import torch
    import dsmvc_gb300 as gb
    from dsmvc_gb300 import synthetic
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    rng = np.random.default_rng(args.seed)
    base_h = int(rng.integers(600, 901))
    frame = synthetic.gray_frame(SWEEP_W, SWEEP_H, synthetic.sweep_width(base_h, SWEEP_W / SWEEP_H),
                                 base_h, seed=args.seed + 1)
    heights = range(SWEEP_HEIGHTS.start, SWEEP_HEIGHTS.stop, args.sweep_step)
    cands = synthetic.native_resolution_candidates(SWEEP_W, SWEEP_H, heights)
    reqs = [r for c in cands for r in (c[3], c[4])]
    dframe = torch.from_numpy(frame).cuda()
    ex = gb.Executor(local)
    stream = torch.cuda.Stream()
    sid = stream.cuda_stream
    torch.cuda.synchronize()

    # Cold: plans built on the host threads, prepared in one upload, the
    # sweep packed, tuned and captured, and run once.  (The device planner
    # gives the same plans; with the geometry, kernel weights and A^T CSR on
    # the host either way, 16 host cores plan C3's 3006 small plans faster
    # than the round trip through the GPU: both timings are reported.)
    t0 = time.perf_counter()
    plans = gb.build_plans(reqs, threads=0)
    t_plan = time.perf_counter() - t0
    pairs = [(plans[2 * i], plans[2 * i + 1]) for i in range(len(cands))]
    ex.prepare_many(plans)
    t1 = time.perf_counter()
    t_upload = t1 - t0 - t_plan
    sweep = gb.Sweep(ex, pairs, dframe.data_ptr(), SWEEP_W, autotune=True, graph=True)
    sweep.run(sid)
    scores = sweep.scores(sid)
    t_cold = time.perf_counter() - t0
    t_prepare = time.perf_counter() - t1
    info = sweep.info()
    th = time.perf_counter()
    device_plans = gb.build_plans(reqs, device=local)
    t_plan_device = time.perf_counter() - th
    del device_plans

    for _ in range(args.warmup):
        sweep.run(sid)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        with torch.cuda.stream(stream):
            start.record(stream)
            for _ in range(args.steps):
                sweep.run(sid)
            stop.record(stream)
        stream.synchronize()
    ms = start.elapsed_time(stop) / args.steps
    warm = len(cands) / (ms / 1e3)

    # End to end: the frame uploaded from pinned host memory and the scores
    # read back every step.
    pinned = torch.from_numpy(frame).pin_memory()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    e2e_steps = max(1, args.steps // 2)
    for _ in range(e2e_steps):
        with torch.cuda.stream(stream):
            dframe.copy_(pinned, non_blocking=True)
        sweep.run(sid)
        scores = sweep.scores(sid)
    e2e = e2e_steps * len(cands) / (time.perf_counter() - t2)

    stages = sweep.profile(sid)
    t3 = time.perf_counter()
    sweep.run_plain(sid)
    plain_scores = sweep.scores(sid)
    plain = len(cands) / (time.perf_counter() - t3)

    # The same sweep with the scoring fused into the columns passes (the
    # descaled planes stay on chip), timed alike.
    sep = gb.Sweep(ex, pairs, dframe.data_ptr(), SWEEP_W, autotune=True, graph=True, fused_scoring=True)
    for _ in range(args.warmup):
        sep.run(sid)
    torch.cuda.synchronize()
    sep_steps = max(1, min(args.steps, 5))
    with torch.cuda.stream(stream):
        start.record(stream)
        for _ in range(sep_steps):
            sep.run(sid)
        stop.record(stream)
    stream.synchronize()
    sep_ms = start.elapsed_time(stop) / sep_steps
    sep_scores = sep.scores(sid)
    sep_info = sep.info()
    sep_stages = sep.profile(sid)
    sep.close()
    # The native resolution shows as the sharpest dip of a kernel's score
    # against its neighbouring heights.  Heights at an exact integer ratio of
    # the source (1080 / 540 here) are left out: there a descale and its
    # re-upscale fit smooth content closely for some kernels whatever the
    # native resolution (Debilinear at 540 dips to 0.67, Debicubic and
    # Delanczos do not dip there).
    dips, by_height = {}, {}
    for k in synthetic.SWEEP_KERNELS:
        idx = [i for i, c in enumerate(cands) if c[0] == k]
        for a, b, c in zip(idx, idx[1:], idx[2:]):
            dips[b] = float(scores[b] / min(scores[a], scores[c]))
            by_height.setdefault(cands[b][2], {})[k] = dips[b]
    best = min((i for i in dips if SWEEP_H % cands[i][2] != 0), key=dips.get)
    base_hits = [i for i, c in enumerate(cands) if c[0] == "bicubic" and c[2] == base_h]
    base_idx = base_hits[0] if base_hits else None

    hbm, peak_kind = peaks()
    # Algorithmic bytes of a step: each candidate's Float32 intermediate
    # (SWEEP_H x its width) written by the rows pass and read by the columns
    # pass, its descaled plane written and read by the scoring, the plans'
    # records and the frame.
    mid_bytes = sum(2 * SWEEP_H * c[1] * 4 for c in cands)
    out_bytes = sum(2 * c[1] * c[2] * 4 for c in cands)
    plan_bytes = sum(int(p.storage_bytes) for p in plans)
    algo = mid_bytes + out_bytes + plan_bytes + frame.nbytes
    achieved = algo / (ms / 1e3) / 1e9
    if rank != 0:
        return
    line = {
        "metric": SWEEP_METRIC, "value": warm, "unit": "candidates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "C3 sweep: 1920x1080 GRAYS f32, heights 500..1000, "
                               "bicubic(0,0.5)/bilinear/lanczos3, mean-L1 score",
                   "candidates": len(cands), "hidden_base_height": base_h,
                   "l2": "per-step intermediates (17 GB) larger than L2; no flush",
                   "parallelism": "replicas"},
        "clocks": clocks.summary(),
        "e2e": {"value": e2e, "unit": "candidates/s", "h2d_bytes_per_step": frame.nbytes,
                "d2h_bytes_per_step": 4 * len(cands)},
        "gpu_launches": info["kernel_launches"] * args.steps,
        "plain_per_candidate": {"value": plain, "unit": "candidates/s",
                                "speedup_batched": warm / plain,
                                "scores_identical": bool(np.array_equal(plain_scores, scores)),
                                "max_rel_diff": float(np.max(np.abs(plain_scores - scores) / np.abs(scores)))},
        "fused_scoring": {"value": len(cands) / (sep_ms / 1e3), "unit": "candidates/s", "ms_per_step": sep_ms,
                          "fused_candidates": sep_info["fused_candidates"], "waves": sep_info["waves"],
                          "device_bytes": sep_info["device_bytes"], "stages_ms": sep_stages,
                          "max_rel_diff_vs_separate": float(np.max(np.abs(sep_scores - scores) / np.abs(scores)))},
        "cold": {"value": len(cands) / t_cold, "unit": "candidates/s", "planning_s": t_plan,
                 "planning": "host planner on all host threads",
                 "planning_device_s": t_plan_device, "plan_upload_s": t_upload,
                 "sweep_setup_s": t_prepare, "seconds": t_cold},
        "sweep": {"waves": info["waves"], "device_bytes": info["device_bytes"],
                  "tune_ms": info["tune_milliseconds"], "segment_rows": info["segment_rows"],
                  "vectors_per_warp": info["vectors_per_warp"],
                  "fused_candidates": info["fused_candidates"],
                  "detected": {"kernel": cands[best][0], "width": cands[best][1],
                               "height": cands[best][2], "score": float(scores[best]),
                               "dip": dips[best]},
                  "found_base_height": cands[best][2] == base_h,
                  "dips_at_detected_height": by_height.get(cands[best][2]),
                  "dips_at_base_height": by_height.get(base_h),
                  "dip_at_base_bicubic": dips.get(base_idx),
                  "stages_ms": stages},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": None, "peak_source": peak_kind,
                     "algorithmic_bytes": algo,
                     "kernel": "whole sweep graph (descale passes, scoring, score reductions)"},
    }
    return line


SERVE_SIZES = [(1280, 720), (1920, 1080), (2560, 1440), (3840, 2160)]
SERVE_KERNELS = [("bilinear", 3, 0.0, 0.5), ("bicubic", 3, 0.0, 0.5), ("lanczos", 3, 0.0, 0.5),
                 ("spline36", 3, 0.0, 0.5)]
SERVE_METRIC = "served Mpix/s with p50/p99 latency (mixed descale requests, Poisson arrivals)"


def run_serving(args, rank, world):
    """Request loop: seeded Poisson arrivals of mixed descale requests --
    sources 1280x720..3840x2160, target ratios from a seeded set of 12 in
    [0.5, 0.9], kernels uniform over bilinear / bicubic(0, 0.5) / lanczos3 /
    spline36, 80 % Float32 (f64mode=0) and 20 % f64mode=2, GRAYS float32 or
    YUV420P16 -- submitted through the server (host frames in pinned memory,
    copies included) at each offered rate for a fixed time."""
    import torch
    import dsmvc_gb300 as gb
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    rng = np.random.default_rng(args.seed)
    ratios = np.sort(rng.uniform(0.5, 0.9, 12))
    ex = gb.Executor(local)
    server = gb.Server(ex, memory_budget=args.serve_budget << 20, streams=args.serve_streams,
                       max_batch=32)

    def even(v):
        v = int(round(v))
        return v + (v & 1)

    # Pinned inputs per (size, format) and output slots per request shape.
    inputs = {}
    for (w, h) in SERVE_SIZES:
        g = torch.empty((h, w), dtype=torch.float32, pin_memory=True).numpy()
        g[...] = np.random.default_rng(w).random((h, w), dtype=np.float32)
        y = [torch.empty((hh, ww), dtype=torch.int16, pin_memory=True).numpy().view(np.uint16)
             for hh, ww in ((h, w), (h // 2, w // 2), (h // 2, w // 2))]
        for k, plane in enumerate(y):
            plane[...] = np.random.default_rng(w + k).integers(4096, 60000, plane.shape, dtype=np.uint16)
        inputs[(w, h)] = (g, y)
    plans = {}
    outputs = {}
    conv_l = gb.integer_conversion(16, False, False)
    conv_c = gb.integer_conversion(16, True, False)

    def plan_pair(sw, sh, ow, oh, kern, f64):
        key = (sw, sh, ow, oh, kern, f64)
        if key not in plans:
            k, taps, b, c = kern
            plans[key] = (gb.AxisPlan(gb.AxisRequest(sw, ow, float(ow), 0.0, k, taps, b, c, 1.0, "symmetric", f64)),
                          gb.AxisPlan(gb.AxisRequest(sh, oh, float(oh), 0.0, k, taps, b, c, 1.0, "symmetric", f64)))
        return plans[key]

    def make_request(i):
        w, h = SERVE_SIZES[int(rng.integers(len(SERVE_SIZES)))]
        ratio = float(ratios[int(rng.integers(len(ratios)))])
        kern = SERVE_KERNELS[int(rng.integers(len(SERVE_KERNELS)))]
        f64 = 2 if rng.random() < 0.2 else 0
        yuv = bool(rng.random() < 0.5)
        dw, dh = even(w * ratio), even(h * ratio)
        g, y = inputs[(w, h)]
        if yuv:
            shapes = [(w, h, dw, dh, y[0], conv_l), (w // 2, h // 2, dw // 2, dh // 2, y[1], conv_c),
                      (w // 2, h // 2, dw // 2, dh // 2, y[2], conv_c)]
        else:
            shapes = [(w, h, dw, dh, g, None)]
        planes = []
        for sw, sh, ow, oh, x, conv in shapes:
            ph, pv = plan_pair(sw, sh, ow, oh, kern, f64)
            slot = (ow, oh, x.dtype.str, i % 48)
            if slot not in outputs:
                t = torch.empty((oh, ow), dtype=torch.float32 if x.dtype == np.float32 else torch.int16,
                                pin_memory=True).numpy()
                outputs[slot] = t if x.dtype == np.float32 else t.view(np.uint16)
            planes.append((ph, pv, x, outputs[slot], conv))
        return planes, sum(sw * sh for sw, sh, *_ in shapes)

    results = []
    clocks = ClockSampler(local, period_ms=100)
    for rate in args.rates:
        # Requests are built (plans planned, output slots pinned) before the
        # clock starts; arrivals follow exponential gaps at `rate` per second.
        count = max(8, int(rate * args.serve_seconds))
        reqs = [make_request(i) for i in range(count)]
        gaps = rng.exponential(1.0 / rate, count)
        # Warm the plan cache and the kernels with every distinct plan once.
        for planes, _ in reqs[:64]:
            server.wait(server.submit(planes))
        server.reset_stats()
        pending = {}
        clocks.__enter__()
        t0 = time.perf_counter()
        due = t0
        for i, ((planes, pix), gap) in enumerate(zip(reqs, gaps)):
            due += gap
            while True:
                now = time.perf_counter()
                if now >= due:
                    break
                time.sleep(min(due - now, 0.0005))
            slot = i % 48
            if slot in pending:                       # the output slot is reused
                server.wait(pending.pop(slot))
            pending[slot] = server.submit(planes)
        for t in pending.values():
            server.wait(t)
        elapsed = time.perf_counter() - t0
        clocks.__exit__(None, None, None)
        st = server.stats()
        results.append({"offered_rate": rate, "requests": count, "seconds": elapsed,
                        "achieved_rate": st["completed"] / elapsed,
                        "mpix_per_s": st["source_pixels"] / elapsed / 1e6,
                        "latency_p50_ms": st["latency_p50_ms"], "latency_p99_ms": st["latency_p99_ms"],
                        "latency_mean_ms": st["latency_mean_ms"], "latency_max_ms": st["latency_max_ms"],
                        "batches": st["batches"], "mean_batch_requests": st["mean_batch_requests"],
                        "failed": st["failed"], "peak_device_bytes": st["peak_device_bytes"]})
    cache = ex.stats()
    server.close()
    if rank != 0:
        return
    head = results[-1]
    line = {
        "metric": SERVE_METRIC, "value": head["mpix_per_s"], "unit": "Mpix/s", "n_gpus": world,
        "steps": len(results), "warmup": 64, "ms_per_step": head["seconds"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic",
        "config": {"workload": "C4 serving: Poisson arrivals, sources 1280x720..3840x2160, ratios "
                               "0.5-0.9, bilinear/bicubic/lanczos3/spline36, 80% f32 / 20% f64mode=2, "
                               "GRAYS f32 or YUV420P16, host frames (pinned)",
                   "memory_budget_mb": args.serve_budget, "streams": args.serve_streams,
                   "l2": "inputs larger than L2 per batch; no flush", "parallelism": "replicas"},
        "latency_p50_ms": head["latency_p50_ms"], "latency_p99_ms": head["latency_p99_ms"],
        "clocks": clocks.summary(),
        "rates": results,
        "plan_cache": {k: cache[k] for k in ("plan_cache_hits", "plan_cache_misses",
                                             "plan_cache_evictions", "plan_cache_bytes")},
        "e2e": {"value": head["mpix_per_s"], "unit": "Mpix/s",
                "note": "every request is a host frame: copies are inside the latency"},
    }
    return line


def _f64_solution(plan_h, plan_v, x):
    """Float64 least-squares descale of `x` (rows x cols) with the plans'
    Float64 weights: (A^T A)^-1 A^T per axis, banded Cholesky solves."""
    import scipy.sparse as sp
    from scipy.linalg import solveh_banded

    def axis(p, data):                       # data: vectors x source
        a = sp.csr_matrix((p.array("transpose_weights_f64"), p.array("transpose_indices"),
                           p.array("transpose_offsets")), shape=(p.destination_size, p.source_size))
        g = (a @ a.T).toarray()
        n, hb = p.destination_size, p.half_bandwidth
        ab = np.zeros((hb + 1, n))
        for d in range(hb + 1):
            ab[hb - d, d:] = np.diagonal(g, d)
        return solveh_banded(ab, (a @ data.T)).T

    y = axis(plan_h, x.astype(np.float64))
    return axis(plan_v, y.T).T


def run_single_frame(args, rank, world):
    """C0: one GRAYS float32 frame, Debicubic(b=0, c=0.5) 1920x1080 ->
    1280x720, padding=3 (symmetric), f64mode=1, on the CPU scalar route (the
    oracle port, one thread) and on the GPU: host-frame call latency, the
    device-resident kernels, and the error against the CPU route and a
    Float64 solve."""
    import torch
    import dsmvc_gb300 as gb
    from dsmvc_gb300 import synthetic
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    sw, sh, dw, dh = 1920, 1080, 1280, 720
    frame = synthetic.gray_frame(sw, sh, dw, dh, seed=args.seed)
    req = lambda s, d, m: gb.AxisRequest(s, d, float(d), 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "symmetric", m)
    h, v = gb.AxisPlan(req(sw, dw, 1)), gb.AxisPlan(req(sh, dh, 1))
    ex = gb.Executor(local)
    ex.prepare(h)
    ex.prepare(v)
    out = np.empty((dh, dw), np.float32)
    for _ in range(args.warmup):
        ex.inverse_2d(h, v, frame, out=out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ex.inverse_2d(h, v, frame, out=out)
    host_ms = (time.perf_counter() - t0) / args.steps * 1e3
    # Device-resident: the same plane from HBM, kernels only.
    dx = torch.from_numpy(frame).cuda()
    dy = torch.empty((dh, dw), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    batch = ex.prepare_batch([gb.PlaneTask(h, v, dx.data_ptr(), sw, dy.data_ptr(), dw, 0, 0, None)])
    for _ in range(args.warmup):
        batch.launch(stream.cuda_stream)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # A single frame takes tens of microseconds: enough steps for a timed
    # region of about 0.3 s, so that the clocks are sampled inside it.
    steps = max(args.steps, 8000)
    with ClockSampler(local) as clocks:
        with torch.cuda.stream(stream):
            start.record(stream)
            for _ in range(steps):
                batch.launch(stream.cuda_stream)
            stop.record(stream)
        stream.synchronize()
    dev_ms = start.elapsed_time(stop) / steps
    gpu = dy.cpu().numpy()
    oh = O.Plan(O.make_request(sw, dw, float(dw), 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "symmetric", 1))
    ov = O.Plan(O.make_request(sh, dh, float(dh), 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "symmetric", 1))
    t1 = time.perf_counter()
    cpu = O.inverse_2d(oh, ov, frame)
    cpu_ms = (time.perf_counter() - t1) * 1e3
    f64 = _f64_solution(gb.AxisPlan(req(sw, dw, 2), cached=False), gb.AxisPlan(req(sh, dh, 2), cached=False),
                        frame)
    pix = sw * sh
    hbm, peak_kind = peaks()
    algo = frame.nbytes + out.nbytes
    if rank != 0:
        return
    line = {
        "metric": "descale Mpix/s, single frame (Debicubic GRAYS 1920x1080->1280x720)",
        "value": pix / (dev_ms / 1e3) / 1e6, "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "device_steps": steps,
        "config": {"workload": "C0: Debicubic(b=0,c=0.5) GRAYS f32 1920x1080->1280x720, padding=3, "
                               "f64mode=1, single frame", "l2": "single 8.3 MB frame (L2-resident)"},
        "clocks": clocks.summary(),
        "e2e": {"value": pix / (host_ms / 1e3) / 1e6, "unit": "Mpix/s", "ms_per_frame": host_ms,
                "h2d_bytes_per_step": frame.nbytes, "d2h_bytes_per_step": out.nbytes},
        "cpu_baseline": {"value": pix / (cpu_ms / 1e3) / 1e6, "unit": "Mpix/s", "cores": 1, "kind": "port",
                         "ms_per_frame": cpu_ms, "sample": "one frame, scalar 2D route"},
        "error": {"max_abs_vs_cpu_scalar": float(np.abs(gpu - cpu).max()),
                  "mean_abs_vs_cpu_scalar": float(np.abs(gpu - cpu).mean()),
                  "max_abs_vs_f64": float(np.abs(gpu - f64).max()),
                  "cpu_scalar_max_abs_vs_f64": float(np.abs(cpu - f64).max())},
        "roofline": {"bound": "hbm", "achieved": algo / (dev_ms / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": algo / (dev_ms / 1e3) / 1e9 / hbm, "traffic": None, "peak_source": peak_kind},
    }
    return line


F64_CASES = {
    "spline64-blur1.1": ("spline64", 3, 0.0, 0.5),
    "bicubic(1/3,1/3)-blur1.1": ("bicubic", 3, 1.0 / 3.0, 1.0 / 3.0),
}


def run_float64(args, rank, world):
    """C2: Despline64 and Debicubic(b=1/3, c=1/3) with blur=1.1, GRAYS
    float32 3840x2160 -> 2560x1440, 32 frames per step, f64mode=2 (forced
    Float64) and f64mode=0 (auto: Float32 for these well-conditioned plans),
    from HBM.  Float64 cases: FLOP/s against the measured FP64 peak; Float32
    cases: compulsory bytes against the HBM peak.  Error against the CPU
    scalar route (float32 ULPs) and a Float64 solve."""
    import torch
    import dsmvc_gb300 as gb
    from dsmvc_gb300 import synthetic
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from common import max_ulp
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    sw, sh, dw, dh = 3840, 2160, 2560, 1440
    nframes = args.frames or 32
    base = synthetic.gray_frame(sw, sh, dw, dh, seed=args.seed)
    rng = np.random.default_rng(args.seed)
    # Eight distinct frames (266 MB, twice the L2) cycled over the step's
    # tasks: a step reads 1.06 GB of inputs.
    distinct = [torch.from_numpy(base + rng.normal(0, 1e-3, base.shape).astype(np.float32)).cuda()
                for _ in range(min(8, nframes))]
    frames = [distinct[i % len(distinct)] for i in range(nframes)]
    outs = [torch.empty((dh, dw), dtype=torch.float32, device="cuda") for _ in range(nframes)]
    fp64_peak = gb.measure_fp64_peak(local)
    hbm, peak_kind = peaks()
    ex = gb.Executor(local)
    stream = torch.cuda.Stream()
    sid = stream.cuda_stream
    x0 = frames[0].cpu().numpy()
    results = {}
    for name, (k, taps, b, c) in F64_CASES.items():
        req = lambda s_, d_, m_: gb.AxisRequest(s_, d_, float(d_), 0.0, k, taps, b, c, 1.1, "symmetric", m_)
        oreq = lambda s_, d_, m_: O.make_request(s_, d_, float(d_), 0.0, k, taps, b, c, 1.1, "symmetric", m_)
        # Float64 solve of the frame with the Float64-retaining plans.
        ref = _f64_solution(gb.AxisPlan(req(sw, dw, 2), cached=False), gb.AxisPlan(req(sh, dh, 2), cached=False),
                            x0)
        for mode in (2, 0):
            h, v = gb.AxisPlan(req(sw, dw, mode), cached=False), gb.AxisPlan(req(sh, dh, mode), cached=False)
            ex.prepare(h)
            ex.prepare(v)
            tasks = [gb.PlaneTask(h, v, frames[i].data_ptr(), sw, outs[i].data_ptr(), dw, 0, 0, None)
                     for i in range(nframes)]
            batch = ex.prepare_batch(tasks)
            for _ in range(args.warmup):
                batch.launch(sid)
            torch.cuda.synchronize()
            start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with ClockSampler(local) as clocks:
                with torch.cuda.stream(stream):
                    start.record(stream)
                    for _ in range(args.steps):
                        batch.launch(sid)
                    stop.record(stream)
                stream.synchronize()
            batch.check(sid)
            ms = start.elapsed_time(stop) / args.steps
            f64 = h.requires_float64 or v.requires_float64
            # Flops per output per axis: 2 per gather entry, 4 per band
            # element (forward and backward multiply-add), 2 for the scale.
            flops = 0
            for p, vectors in ((h, sh), (v, dw)):
                flops += vectors * (2 * int(p.nonzeros) + p.destination_size * (4 * p.half_bandwidth + 2))
            flops *= nframes
            gpu = outs[0].cpu().numpy()
            cpu = O.inverse_2d(O.Plan(oreq(sw, dw, mode)), O.Plan(oreq(sh, dh, mode)), x0)
            algo = nframes * (sw * sh + dw * dh) * 4
            results[f"{name}/f64mode={mode}"] = {
                "route": "float64" if f64 else "float32", "ms_per_step": ms,
                "mpix_per_s": nframes * sw * sh / (ms / 1e3) / 1e6,
                "gflops": flops / (ms / 1e3) / 1e9,
                "fp64_frac": (flops / (ms / 1e3) / 1e12 / fp64_peak) if f64 else None,
                "hbm_frac": algo / (ms / 1e3) / 1e9 / hbm,
                "rcond": [h.normal_rcond, v.normal_rcond], "half_bandwidth": [h.half_bandwidth, v.half_bandwidth],
                "max_ulp_vs_cpu_scalar": max_ulp(gpu, cpu),
                "max_abs_vs_cpu_scalar": float(np.abs(gpu - cpu).max()),
                "mean_abs_vs_cpu_scalar": float(np.abs(gpu - cpu).mean()),
                "max_abs_vs_f64": float(np.abs(gpu - ref).max()),
                "cpu_scalar_max_abs_vs_f64": float(np.abs(cpu - ref).max()),
                "clocks": clocks.summary(),
                "gpu_launches": batch.info()["kernel_launches"] * args.steps,
            }
            if f64:
                # The kernels in the CPU scalar route's operation order
                # (unfused, true division), for comparison.
                os.environ["DSMVC_GB_F64_EXACT"] = "1"
                try:
                    exact_ex = gb.Executor(local)
                finally:
                    del os.environ["DSMVC_GB_F64_EXACT"]
                exact_ex.prepare(h)
                exact_ex.prepare(v)
                eb = exact_ex.prepare_batch(tasks)
                for _ in range(2):
                    eb.launch(sid)
                torch.cuda.synchronize()
                start.record(stream)
                for _ in range(max(3, args.steps // 4)):
                    eb.launch(sid)
                stop.record(stream)
                stream.synchronize()
                ems = start.elapsed_time(stop) / max(3, args.steps // 4)
                eb.check(sid)
                egpu = outs[0].cpu().numpy()
                results[f"{name}/f64mode={mode}"]["cpu_order"] = {
                    "ms_per_step": ems, "fp64_frac": flops / (ems / 1e3) / 1e12 / fp64_peak,
                    "max_ulp_vs_cpu_scalar": max_ulp(egpu, cpu), "speedup_of_fused": ems / ms}
                del eb
                exact_ex.close()
            del batch
    if rank != 0:
        return None
    head = results["spline64-blur1.1/f64mode=2"]
    f32 = results["bicubic(1/3,1/3)-blur1.1/f64mode=0"]
    line = {
        "metric": "descale Mpix/s, Float64 route (Despline64 blur 1.1, GRAYS 3840x2160->2560x1440)",
        "value": head["mpix_per_s"], "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"C2: GRAYS f32 3840x2160->2560x1440, {nframes} frames, blur 1.1, "
                               "f64mode 2 and 0", "frames_per_step": nframes,
                   "l2": f"inputs ({nframes * sw * sh * 4 / 1e9:.2f} GB per step from 8 distinct "
                         "frames of 266 MB) larger than L2; no flush"},
        "clocks": head["clocks"],
        "fp64_peak_tflops": fp64_peak, "cases": results,
        "roofline": {"bound": "fp64", "achieved": head["gflops"] / 1e3, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": head["fp64_frac"], "traffic": None,
                     "peak_source": "measured (dsmvc_gb_measure_fp64_peak)"},
        "roofline_f32_debicubic": {"bound": "hbm", "achieved": f32["hbm_frac"] * hbm, "peak": hbm,
                                   "unit": "GB/s", "frac": f32["hbm_frac"], "peak_source": peak_kind,
                                   "case": "bicubic(1/3,1/3)-blur1.1/f64mode=0 (Float32 route)"},
    }
    return line


SUB_WORKLOADS = {"c0": run_single_frame, "c2": run_float64, "c3": run_sweep, "c4": run_serving}


def run_configs(args, rank, world):
    """The other configurations, each measured as its own line (own timed
    region, clocks and error figures) and nested in the headline line:
    c0 single frame, c2 4K Float64/Float32, c3 candidate sweep, c4 request
    loop.  Shorter runs than the standalone --workload lines."""
    import torch
    sub = argparse.Namespace(**vars(args))
    sub.steps = max(3, min(args.steps, 20))
    sub.warmup = 3
    sub.frames = None
    sub.rates = [200.0, 800.0]
    sub.serve_seconds = 2.0
    out = {}
    for key, fn in SUB_WORKLOADS.items():
        t0 = time.perf_counter()
        try:
            out[key] = fn(sub, rank, world) or {}
        except Exception as e:  # noqa: BLE001 - recorded in the line, the headline stands
            out[key] = {"error": f"{type(e).__name__}: {e}"}
        out[key]["wall_s"] = time.perf_counter() - t0
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return out


def c1_error(frame, outputs, plans, convs):
    """Error of the step's first frame, luma and one chroma plane (computed
    outside the timed region): codes against the CPU scalar route (the
    reference engine built on this machine, else the oracle port) and
    against an unrounded Float64 solve of the same plane in code units."""
    import dsmvc_gb300 as gb
    O, R = checker_modules()
    res = {}
    for name, idx, (hk, vk), conv in (("luma", 0, ("luma_h", "luma_v"), convs[0]),
                                      ("chroma_u", 1, ("chroma_h", "chroma_v"), convs[1])):
        x = frame[idx]
        got = outputs[idx].astype(np.int64)
        hq, vq = plans[hk].request, plans[vk].request
        oreq = lambda q: O.make_request(q.source_size, q.destination_size, q.active_length, q.shift,
                                        q.kernel, q.taps, q.b, q.c, q.blur, q.border, q.f64_mode)
        if R is not None:
            cpu = R.inverse_2d(R.Plan(oreq(hq)), R.Plan(oreq(vq)), x, conv, path=0)
        else:
            cpu = O.inverse_2d(O.Plan(oreq(hq)), O.Plan(oreq(vq)), x, conv)
        f64p = lambda q: gb.AxisPlan(gb.AxisRequest(q.source_size, q.destination_size, q.active_length,
                                                    q.shift, q.kernel, q.taps, q.b, q.c, q.blur,
                                                    q.border, 2), cached=False)
        xf = (x.astype(np.float64) - conv[0]) * conv[1]
        ref = _f64_solution(f64p(hq), f64p(vq), xf) * conv[2] + conv[3]
        res[name] = {"max_codes_vs_cpu_scalar": int(np.max(np.abs(got - cpu.astype(np.int64)))),
                     "mismatched_samples_vs_cpu_scalar": int(np.count_nonzero(got != cpu)),
                     "max_abs_codes_vs_f64": float(np.max(np.abs(got - ref))),
                     "cpu_scalar_max_abs_codes_vs_f64": float(np.max(np.abs(cpu.astype(np.int64) - ref)))}
    res["checker"] = "reference engine (scalar route)" if R is not None else "oracle port (scalar route)"
    return res


def workload_config():
    return {"workload": "Delanczos(taps=3) YUV420P16 1920x1080->1440x810, 64 frames, "
                        "f64mode=0, padding=1",
            "frames_per_step": FRAMES, "planes_per_frame": 3,
            "source_pixels_per_step": pixels_per_frame() * FRAMES,
            "l2": "inputs (398 MB) larger than L2; no flush", "parallelism": "replicas"}


def pageable_frames(ex, gb, calls, pix_step, steps):
    """The same multi-plane call with the step's frames in ordinary
    (pageable) host memory, one ring per direction as a frame pool would
    hold them: as they are, and after the host block registry has
    page-locked both rings (reported twice, within a 1 GiB limit)."""
    total_in = sum(c[2].size for c in calls)
    total_out = sum(c[4].size for c in calls)
    ring_in = np.empty(total_in, np.uint16)
    ring_out = np.empty(total_out, np.uint16)
    planes, at_in, at_out = [], 0, 0
    for h, v, pin, conv, pout in calls:
        src = ring_in[at_in:at_in + pin.size].reshape(pin.shape)
        src[...] = pin
        dst = ring_out[at_out:at_out + pout.size].reshape(pout.shape)
        at_in += pin.size
        at_out += pout.size
        planes.append((h, v, src, dst, conv))

    def rate():
        run = ex.host_planes(planes)
        run.run()   # warm-up
        t0 = time.perf_counter()
        for _ in range(steps):
            run.run()
        return steps * pix_step / (time.perf_counter() - t0) / 1e6

    plain = rate()
    hb = gb.host_blocks
    owner = id(ring_in)
    hb.set_limit(owner, 1 << 30)
    s0 = hb.stats()
    for _ in range(2):
        hb.note_array(owner, ring_in)
        hb.note_array(owner, ring_out)
    registered = hb.covered(ring_in.ctypes.data, ring_in.nbytes) and hb.covered(ring_out.ctypes.data, ring_out.nbytes)
    fast = rate() if registered else None
    s1 = hb.stats()
    hb.drop_owner(owner)
    return {"unit": "Mpix/s", "unregistered": plain, "registered": fast,
            "registrations": s1["registrations"] - s0["registrations"],
            "api": "dsmvc_gb_inverse_2d_planes after dsmvc_gb_host_blocks_note_use (second use registers)"}


def native_host_calls(gb, reqs, convs, frames, threads=16, steps=10):
    """The per-plane synchronous calls of the step from `threads` C++
    threads straight into the C ABI (bench_host_calls.cpp, compiled here
    against the in-tree library): the plugin's calling pattern with no
    Python between the threads and the library.  The Python-thread figure
    beside it is bound by the binding's own per-call time, which holds the
    interpreter lock."""
    import shutil
    import tempfile
    here = os.path.dirname(os.path.abspath(__file__))
    gxx = shutil.which("g++")
    if not gxx:
        return {"unavailable": "no g++ on this host"}
    libdir = os.path.dirname(gb.LIB_PATH)

    def req_arg(q):
        c = q.to_c()
        return ",".join(repr(getattr(c, f)) for f, _ in c._fields_)

    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "bench_host_calls")
        r = subprocess.run([gxx, "-std=c++20", "-O2", "-pthread", "-I", os.path.join(here, "include"),
                            os.path.join(here, "bench_host_calls.cpp"), "-L", libdir, "-ldsmvc_gb300",
                            f"-Wl,-rpath,{libdir}", "-o", exe], capture_output=True, text=True)
        if r.returncode != 0:
            return {"unavailable": "compiling bench_host_calls.cpp failed: "
                    + ((r.stderr.strip().splitlines() or ["?"])[-1])[:200]}
        args = [exe, str(threads), str(steps), str(frames)]
        args += [req_arg(reqs[k]) for k in ("luma_h", "luma_v", "chroma_h", "chroma_v")]
        args += [",".join(repr(x) for x in cv) for cv in convs]
        r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    try:
        out = json.loads((r.stdout.strip().splitlines() or ["{}"])[-1])
    except ValueError:
        out = {"error": (r.stdout + r.stderr).strip()[-200:]}
    if "mpix_s" in out:
        out = {"value": out["mpix_s"], "unit": "Mpix/s", **out,
               "api": "dsmvc_gb_inverse_2d_u16 per plane from C++ threads (bench_host_calls.cpp)"}
    return out


def main():
    global FRAMES
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--frames", type=int, default=None,
                    help="frames per step (profiling runs use fewer; the benchmark lines use 64, "
                         "and 32 for c2)")
    ap.add_argument("--workload", default="c1", choices=["c0", "c1", "c2", "c3", "c4"],
                    help="c1: Delanczos YUV420P16 frames (default); c0: one Debicubic GRAYS frame; "
                         "c2: Float64 route at 4K; c3: candidate sweep; c4: request loop")
    ap.add_argument("--rates", type=float, nargs="+", default=[200.0, 800.0],
                    help="c4: offered request rates (per second)")
    ap.add_argument("--serve-seconds", type=float, default=3.0)
    ap.add_argument("--serve-budget", type=int, default=8192, help="c4: arena MiB")
    ap.add_argument("--serve-streams", type=int, default=4)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--sweep-step", type=int, default=1,
                    help="c3: height step (1 = the full sweep; larger steps give small profiling cases)")
    ap.add_argument("--kernels-only", action="store_true",
                    help="skip the end-to-end and CPU legs and the other configurations (profiling runs)")
    ap.add_argument("--no-configs", action="store_true",
                    help="headline line only (no c0/c2/c3/c4 blocks)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    FRAMES = args.frames or FRAMES

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if args.workload != "c1" and args.impl != "reference":
        line = SUB_WORKLOADS[args.workload](args, rank, world)
        if line is not None:
            print(json.dumps(line), flush=True)
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return

    import dsmvc_gb300 as gb
    torch.cuda.set_device(local)
    ex = gb.Executor(local)
    reqs = plane_requests(gb)
    plans = {k: gb.AxisPlan(r) for k, r in reqs.items()}
    for p in plans.values():
        ex.prepare(p)
    ex.seal()
    assert not any(p.requires_float64 for p in plans.values())
    luma_conv = gb.integer_conversion(16, chroma=False, full_range=False)
    chroma_conv = gb.integer_conversion(16, chroma=True, full_range=False)

    frames = make_frames(product_arrays(gb), 8, 20250 + rank)  # 8 distinct frames, reused cyclically
    stream = torch.cuda.Stream()
    dev_in, dev_out, tasks = [], [], []
    for f in range(FRAMES):
        for idx, plane in enumerate(frames[f % len(frames)]):
            hk, vk, conv = ("luma_h", "luma_v", luma_conv) if idx == 0 else \
                ("chroma_h", "chroma_v", chroma_conv)
            h, v = plans[hk], plans[vk]
            x = torch.from_numpy(plane.view(np.int16)).cuda()
            y = torch.empty((v.destination_size, h.destination_size), dtype=torch.int16,
                            device="cuda")
            dev_in.append(x)
            dev_out.append(y)
            tasks.append(gb.PlaneTask(h, v, x.data_ptr(), h.source_size, y.data_ptr(),
                                      h.destination_size, 2, 0, conv))
    torch.cuda.synchronize()
    sid = stream.cuda_stream
    # The step's 192 planes are routed and uploaded once; each step then
    # issues only the kernels.
    batch = ex.prepare_batch(tasks)
    for _ in range(args.warmup):
        batch.launch(sid)
    torch.cuda.synchronize()
    batch.check(sid)
    launches0 = ex.stats()["launches"]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        with torch.cuda.stream(stream):
            start.record(stream)
            for _ in range(args.steps):
                batch.launch(sid)
            stop.record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    batch.check(sid)
    elapsed_ms = start.elapsed_time(stop)
    launches = ex.stats()["launches"] - launches0
    # Per-kernel event times and algorithmic bytes, from the same steps run
    # again outside the timed region (events between kernels stay out of the
    # timed number).
    ex.profile(True)
    with torch.cuda.stream(stream):
        for _ in range(args.steps):
            batch.launch(sid)
    torch.cuda.synchronize()
    ktimes = ex.kernel_times()
    ex.profile(False)
    elapsed_ms = max_over_ranks(elapsed_ms, dist, "cuda")
    pix_step = pixels_per_frame() * FRAMES
    value = whole_job_rate(pix_step, world, args.steps, elapsed_ms)

    # End to end: the step's 192 host planes (pinned) through the pipelined
    # multi-plane host call of the C ABI (uploads, kernels and downloads of
    # successive plane groups overlap); also the per-plane synchronous calls
    # from 16 caller threads (the plugin's frame-parallel requests).
    # The frames live in one pinned ring per direction, plane after plane
    # (as a frame server's buffer pool would hold them).
    host_in, host_out, calls = [], [], []
    layout = []
    for f in range(0 if args.kernels_only else FRAMES):
        for idx, plane in enumerate(frames[f % len(frames)]):
            hk, vk, conv = ("luma_h", "luma_v", luma_conv) if idx == 0 else \
                ("chroma_h", "chroma_v", chroma_conv)
            layout.append((plane, plans[hk], plans[vk], conv))
    if layout:
        ring_in = torch.empty(sum(pl.size for pl, _, _, _ in layout), dtype=torch.int16,
                              pin_memory=True).numpy().view(np.uint16)
        ring_out = torch.empty(sum(v.destination_size * h.destination_size for _, h, v, _ in layout),
                               dtype=torch.int16, pin_memory=True).numpy().view(np.uint16)
        at_in = at_out = 0
        for plane, h, v, conv in layout:
            pin = ring_in[at_in:at_in + plane.size].reshape(plane.shape)
            pin[...] = plane
            out = ring_out[at_out:at_out + v.destination_size * h.destination_size].reshape(
                v.destination_size, h.destination_size)
            at_in += plane.size
            at_out += out.size
            host_in.append(pin)
            host_out.append(out)
            calls.append((h, v, pin, conv, out))
    h2d = sum(a.nbytes for a in host_in)
    d2h = sum(a.nbytes for a in host_out)

    def call(c):
        ex.inverse_2d(c[0], c[1], c[2], c[3], out=c[4])

    e2e = e2e_calls = None
    if calls:
        planes = ex.host_planes([(c[0], c[1], c[2], c[4], c[3]) for c in calls])
        planes.run()  # warm-up
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            planes.run()
        e2e_s = time.perf_counter() - t0
        e2e = world * args.e2e_steps * pix_step / e2e_s / 1e6
        with cf.ThreadPoolExecutor(max_workers=16) as pool:
            list(pool.map(call, calls))  # warm-up
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                list(pool.map(call, calls))
            e2e_calls = world * args.e2e_steps * pix_step / (time.perf_counter() - t0) / 1e6
    link = link_bandwidth(h2d, d2h) if calls else None
    pageable = pageable_frames(ex, gb, calls, pix_step * world, args.e2e_steps) if calls else None
    native = native_host_calls(gb, reqs, (luma_conv, chroma_conv), FRAMES) if calls and world == 1 else None

    hbm, peak_kind = peaks()
    total_ms = sum(k["milliseconds"] for k in ktimes)
    total_bytes = sum(k["bytes"] for k in ktimes)
    dominant = max(ktimes, key=lambda k: k["milliseconds"]) if ktimes else None
    step_bytes = total_bytes / max(1, args.steps)
    achieved = step_bytes / (elapsed_ms / args.steps / 1e3) / 1e9 if elapsed_ms else 0.0

    if rank != 0:
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu_baseline and not args.kernels_only and world == 1:
        threads, how = host_threads()
        cpu = dict(cpu_baseline(frames, threads, budget_s=args.cpu_seconds), cores_source=how)
    err = None
    if not args.kernels_only and world == 1:
        err = c1_error(frames[0], [dev_out[i].cpu().numpy().view(np.uint16) for i in range(2)],
                       plans, (luma_conv, chroma_conv))
    line = {
        "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(),
        "clocks": clocks.summary(),
        "e2e": {"value": e2e, "unit": "Mpix/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "api": "dsmvc_gb_inverse_2d_planes (192 planes in one pinned ring per direction)",
                "per_plane_calls_16_threads": e2e_calls,
                "per_plane_calls_16_native_threads": native,
                "link": link,
                "link_frac": (((h2d + d2h) / (pix_step / (e2e * 1e6)) / 1e9) / link["concurrent_gbs"])
                if link and e2e else None,
                "pageable_frames": pageable},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm,
                     "traffic": DRAM_BYTES_PER_FRAME * FRAMES,
                     "traffic_source": TRAFFIC_SOURCE,
                     "algorithmic_bytes": step_bytes,
                     "peak_source": peak_kind,
                     "kernel": "2D descale step (horizontal + vertical passes of 192 planes, "
                               "two overlapping parts); achieved = algorithmic bytes / step time",
                     "batch_parts": batch.info()["parts"],
                     "kernel_ms_sum_per_step": total_ms / max(1, args.steps),
                     "kernels": [dict(k, share=k["milliseconds"] / total_ms) for k in ktimes],
                     "dominant": dominant["name"] if dominant else None},
        "cpu_baseline": cpu,
        "error": err,
    }
    if not args.kernels_only and not args.no_configs and world == 1:
        line["configs"] = run_configs(args, rank, world)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
