"""Benchmark of the GB300 3DGS forward path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl gsr|reference]

Default workload: ``serve_mix``, a stream of 512 render requests (Poisson
arrivals at 240/s) over resident scenes of 0.5, 2, 5 and 10 M Gaussians at
720p-2160p, served by continuous batching against the plain per-request
forward; a step is one request, and the line also carries a plain_3m_1080p
plain-forward measurement.

Plain-forward workloads (``plain_3m_1080p``: 3,000,000 Gaussians, clustered
with a heavy-tailed scale distribution, 1920x1080, fx=fy=1400, 16x16 tiles,
FP16 SH, the reference's E2E variant ``preranges_smem_persistent_lite_e2e``;
also ``city_20m_8k``, ``clustered_1m_1080p``, ``plain_100k_800x600``): a step
is one frame (preprocess -> tile-key radix sort -> tile ranges -> persistent
blend).

value     frames/s, device-timed over K back-to-back frames (CUDA events on
          the launching stream; inputs resident in HBM; the scenes are larger
          than L2, so no flush is needed between frames).
e2e       frames/s through the public drop-in API (Rasterizer.forward with
          the host-read camera/background, status read-back and the frame
          copied to pinned host memory every step).
roofline  the dominant kernel of the frame, timed live with CUDA events
          recorded between stages on the launching stream.
cpu_baseline  the FP64 CPU oracle (oracle/), multithreaded, on whole frames.

``gather_plain_3m_1080p`` times the feature gather (gather_features) alone,
over the sorted list of one plain_3m_1080p frame: GB/s of algorithmic bytes.

--impl reference runs the reference's CPU arm: the reference ships no CPU
path, so this is the FP64 oracle restatement of its algorithm on all host
cores.  Multi-GPU: replicas only (one independent renderer per rank).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

E2E_VARIANT = "preranges_smem_persistent_lite_e2e"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps: frames (plain-forward workloads, default 500) or saturated passes over the "
                         "request stream (serve_mix, default 10)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="serve_mix",
                    help="serve_mix (the served stream, the headline), or a plain-forward workload: plain_3m_1080p, "
                         "plain_100k_800x600, clustered_1m_1080p, city_20m_8k; diff_1m_8cam (forward + "
                         "backward); gather_plain_3m_1080p, prepare_plain_3m (the feature gather or the scene "
                         "transform alone)")
    ap.add_argument("--impl", default="gsr", choices=["gsr", "reference", "reference-gpu"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true",
                    help="device-timed frames only (no e2e, CPU baseline or reference pipeline): for profiling")
    ap.add_argument("--cap-log2", type=int, default=0, help="key-buffer capacity 2^n (default: by scene size)")
    ap.add_argument("--serve-profile", default=None, metavar="JSON",
                    help="serve_mix only: skip the plain arm and the autotuner, serve the stream with this "
                         "TuneConfig (JSON, e.g. the bench line's config.tuned) twice to warm up and once more "
                         "inside the NVTX range 'timed', device-only: for ncu launch lists")
    ap.add_argument("--diff-profile", action="store_true",
                    help="diff_1m_8cam only: after three warm-up steps of each path, run one step through "
                         "render_views inside the NVTX start/end range 'timed_views' and one with a pass per "
                         "camera inside 'timed_loop': for ncu launch lists")
    ap.add_argument("--pipeline", default="single", choices=["single", "depth_first"],
                    help="single-pass 64-bit key sort, or depth sort + 32-bit tile sort")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, dist, device) -> float:
    """The largest of every rank's value (timings are reported for the slowest
    replica); the value itself on one process."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- peaks
def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def committed_traffic(workload: str, kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(workload, {}).get(kernel)
    except (OSError, ValueError):
        return None


# ----------------------------------------------------------------------------- CPU arm
def cpu_frames(raw, cam, seconds: float, half: bool = True):
    """Time the FP64 oracle on whole frames for about `seconds`."""
    import numpy as np

    from oracle import oracle as O

    op, cov = O.scene_transform(raw.log_scales, raw.quats, raw.opacity_logits)
    threads = O.nthreads_default()
    n, t0 = 0, time.perf_counter()
    while True:
        O.forward(raw.means, raw.shs, op, cov, cam, cadence=16, half_sh=half, nthreads=threads)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= 50:
            break
    return n / el, threads, n, el


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from polysplat_gb300 import scenes

    if args.workload == "serve_mix":
        # the request stream in order on the host cores (the reference has
        # no CPU path: its algorithm restated in FP64), bounded to about a minute
        raws, reqs = scenes.serve_mix()
        cpu = serve_cpu_baseline(raws, reqs[:CPU_SAMPLE_REQUESTS], seconds=60.0)
        line = {"impl": "reference", "metric": "frames/s", "value": cpu["value"], "unit": "frames/s",
                "n_gpus": world, "steps": cpu["requests"], "warmup": 0,
                "step": "one request of the stream, on the host cores (a bounded sample: its first %d requests)"
                        % CPU_SAMPLE_REQUESTS,
                "ms_per_step": 1000.0 / cpu["value"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": serve_config(raws, reqs, world),
                "cpu_baseline": cpu,
                "e2e": {"value": cpu["value"], "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0
    raw, cams = scenes.workload(args.workload)
    cam = cams[0]
    from oracle import oracle as O

    op, cov = O.scene_transform(raw.log_scales, raw.quats, raw.opacity_logits)
    threads = O.nthreads_default()
    for _ in range(max(0, min(args.warmup, 1))):
        O.forward(raw.means, raw.shs, op, cov, cam, cadence=16, half_sh=True, nthreads=threads)
    steps = max(1, min(args.steps, 8))
    t0 = time.perf_counter()
    for _ in range(steps):
        O.forward(raw.means, raw.shs, op, cov, cam, cadence=16, half_sh=True, nthreads=threads)
    el = time.perf_counter() - t0
    fps = steps / el
    line = {"impl": "reference", "metric": "frames/s", "value": fps, "unit": "frames/s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1000.0 * el / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "width": cam.width, "height": cam.height,
                       "gaussians": raw.num, "variant": E2E_VARIANT},
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": threads, "kind": "port",
                             "sample": "%d whole frames of %s (FP64 oracle restatement; the reference ships no "
                                       "CPU render path)" % (steps, args.workload)},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- GPU arm
def run_gsr(args):
    import torch

    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist = dist_mod
        dist.init_process_group("nccl", rank=rank, world_size=world)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.workload == "serve_mix" and args.serve_profile:
        line = run_serve_profile(args, dev)
    elif args.workload == "serve_mix":
        line = run_serve(args, dev, rank, world, dist)
    elif args.workload == "diff_1m_8cam":
        line = run_diff(args, dev, rank, world, dist)
    elif args.workload == "gather_plain_3m_1080p":
        line = run_gather(args, dev, rank, world, dist)
    elif args.workload == "prepare_plain_3m":
        line = run_prepare(args, dev, rank, world, dist)
    else:
        line = forward_line(args, dev, rank, world, dist)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def forward_line(args, dev, rank, world, dist):
    """The plain forward of one workload: device-timed frames/s, stage times,
    roofline, e2e through the public API, CPU and reference-GPU arms."""
    import ctypes

    import numpy as np
    import torch

    from polysplat_gb300 import Camera, Rasterizer, Scene, ops, scenes
    from polysplat_gb300._lib import check, lib

    raw, cams = scenes.workload(args.workload)
    cam_spec = cams[0]
    scene = Scene.from_raw(raw, dev)
    cam = Camera.from_spec(cam_spec)
    cap = 1 << (args.cap_log2 or (28 if raw.num > 10_000_000 else 26))
    rast = Rasterizer(scene, cap, 1 << 18)
    bg = torch.zeros(3)

    # ---- device-timed value: the fused forward through the C ABI (no host sync per frame)
    L = lib()
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    cam_pos = (ctypes.c_float * 3)(*cam.position.tolist())
    cam_rot = (ctypes.c_float * 9)(*cam.rotation.reshape(-1).tolist())
    bgc = (ctypes.c_float * 3)(0.0, 0.0, 0.0)
    out = torch.zeros((cam.height, cam.width, 3), dtype=torch.uint8, device=dev)
    ws = rast.list_sorting_space
    wsb = ws.numel()

    df = args.pipeline == "depth_first"
    scratch = None
    if df:
        scratch = torch.zeros(ops.depth_first_scratch_size(scene.num_vertex), dtype=torch.int8, device=dev)

    def frame_df():
        st = L.gsr_forward_depth_first(
            1, scene.num_vertex, scene.position.data_ptr(), scene.shs_half.data_ptr(), 1, scene.opacity.data_ptr(),
            scene.cov3d.data_ptr(), cam.width, cam.height, 16, 16, cam_pos, cam_rot, cam.focal_x, cam.focal_y,
            cam.zFar, cam.zNear, rast.curr_offset.data_ptr(), ws.data_ptr(), wsb, scratch.data_ptr(),
            scratch.numel(), rast.gaussian_keys_unsorted.data_ptr(), rast.gaussian_values_unsorted.data_ptr(),
            rast.gaussian_keys_sorted.data_ptr(), rast.gaussian_values_sorted.data_ptr(), cap,
            rast.points_xy.data_ptr(), rast.rgb_depth.data_ptr(), rast.conic_opacity.data_ptr(), None, bgc,
            out.data_ptr(), sh)
        check(st, "forward_depth_first")

    def frame_single():
        st = L.gsr_forward(1, scene.num_vertex, scene.position.data_ptr(), scene.shs_half.data_ptr(), 1,
                           scene.opacity.data_ptr(), scene.cov3d.data_ptr(), cam.width, cam.height, 16, 16, cam_pos,
                           cam_rot, cam.focal_x, cam.focal_y, cam.zFar, cam.zNear, rast.curr_offset.data_ptr(),
                           ws.data_ptr(), wsb, rast.gaussian_keys_unsorted.data_ptr(),
                           rast.gaussian_values_unsorted.data_ptr(), rast.gaussian_keys_sorted.data_ptr(),
                           rast.gaussian_values_sorted.data_ptr(), cap, rast.points_xy.data_ptr(),
                           rast.rgb_depth.data_ptr(), rast.conic_opacity.data_ptr(), None, bgc, out.data_ptr(), sh)
        check(st, "forward")

    frame = frame_df if df else frame_single
    for _ in range(max(3, args.warmup)):
        frame()
    num = ops._read_status(ws, rast.curr_offset, cap, "forward")
    tiles = ((cam.width + 15) // 16) * ((cam.height + 15) // 16)
    end_bit = 32 + tiles.bit_length()
    passes = (end_bit + 7) // 8
    tile_passes = (tiles.bit_length() + 7) // 8

    # stage events recorded by the library: [preprocess, upsweep, pass 0..passes-1, render]
    K = args.steps
    check(L.gsr_profile_begin(K), "profile_begin")

    sampler = ClockSampler(dev.index or 0)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(K):
        frame()
    t_end.record(stream)
    torch.cuda.synchronize()
    MAXS = 16
    ms_buf = (ctypes.c_float * (K * MAXS))()
    n_stages = L.gsr_profile_read(ms_buf, K, MAXS)
    L.gsr_profile_end()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    elapsed_ms = t_start.elapsed_time(t_end)
    elapsed_ms = max_over_ranks(elapsed_ms, dist, dev)
    fps = world * K / (elapsed_ms / 1000.0)

    if df:
        stage_names = (["preprocess", "compact", "depth_upsweep"] + ["depth_pass%d" % p for p in range(4)]
                       + ["offsets", "emit", "tile_upsweep"] + ["tile_pass%d" % p for p in range(tile_passes)]
                       + ["tile_ranges", "render"])
    else:
        stage_names = (["preprocess", "sort_upsweep"] + ["sort_pass%d" % p for p in range(passes)]
                       + ["tile_ranges", "render"])
    if n_stages != len(stage_names):
        raise RuntimeError("expected %d timed stages, the library recorded %d" % (len(stage_names), n_stages))
    stage_avg = {nm: statistics.mean(ms_buf[f * MAXS + i] for f in range(K)) for i, nm in enumerate(stage_names)}
    # passes the depth compression made unnecessary return at once
    pass_key = "tile_pass" if df else "sort_pass"
    pass_ms = [stage_avg["%s%d" % (pass_key, p)] for p in range(tile_passes if df else passes)]
    working = [t for t in pass_ms if t > 0.2 * max(pass_ms)]
    pass_avg = statistics.mean(working)

    # algorithmic bytes per launch: every byte the kernel must move once
    P = scene.num_vertex
    peak, peak_kind = measured_peaks()
    # a digit pass reads and writes every (key, value) pair: 12-byte pairs in
    # the single-pass sort, 8-byte (tile id, value) pairs in the depth-first one
    pass_bytes = (16.0 if df else 24.0) * num
    # preprocess: scene read + features of emitters + keys (the counting pass
    # writes 32 B of per-Gaussian records instead of keys)
    pre_bytes = P * (12 + 4 + 24 + 96) + (P * 32 if df else num * 12)
    cand = {"k_pass": (pass_avg, pass_bytes), "k_preprocess": (stage_avg["preprocess"], pre_bytes)}
    dom = max(cand, key=lambda k: cand[k][0] * (len(working) if k == "k_pass" else 1))
    dur_ms, abytes = cand[dom]
    achieved = abytes / (dur_ms / 1000.0) / 1e9
    traffic = committed_traffic(args.workload, dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                "algorithmic_bytes": abytes, "avg_launch_ms": dur_ms}

    # ---- the same frame with quad keys (one key per 2x2 group of tiles; same image)
    quad = None
    if not df:
        from polysplat_gb300._lib import QUAD_KEYS

        img_tile = out.clone()

        def frame_quad():
            st = L.gsr_forward(1 | QUAD_KEYS, scene.num_vertex, scene.position.data_ptr(),
                               scene.shs_half.data_ptr(), 1, scene.opacity.data_ptr(), scene.cov3d.data_ptr(),
                               cam.width, cam.height, 16, 16, cam_pos, cam_rot, cam.focal_x, cam.focal_y, cam.zFar,
                               cam.zNear, rast.curr_offset.data_ptr(), ws.data_ptr(), wsb,
                               rast.gaussian_keys_unsorted.data_ptr(), rast.gaussian_values_unsorted.data_ptr(),
                               rast.gaussian_keys_sorted.data_ptr(), rast.gaussian_values_sorted.data_ptr(), cap,
                               rast.points_xy.data_ptr(), rast.rgb_depth.data_ptr(), rast.conic_opacity.data_ptr(),
                               None, bgc, out.data_ptr(), sh)
            check(st, "forward (quad keys)")

        for _ in range(max(3, args.warmup)):
            frame_quad()
        num_q = ops._read_status(ws, rast.curr_offset, cap, "forward (quad keys)")
        same = bool(torch.equal(out, img_tile))
        Kq = max(10, K // 2)
        check(L.gsr_profile_begin(Kq), "profile_begin")
        qa, qb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        qa.record(stream)
        for _ in range(Kq):
            frame_quad()
        qb.record(stream)
        torch.cuda.synchronize()
        qbuf = (ctypes.c_float * (Kq * MAXS))()
        nq = L.gsr_profile_read(qbuf, Kq, MAXS)
        L.gsr_profile_end()
        q_ms = qa.elapsed_time(qb) / Kq
        qpasses = nq - 4 if nq > 4 else 0
        qnames = ["preprocess", "sort_upsweep"] + ["sort_pass%d" % p for p in range(qpasses)] + ["tile_ranges",
                                                                                                  "render"]
        q_stages = ({nm: statistics.mean(qbuf[f * MAXS + i] for f in range(Kq)) for i, nm in enumerate(qnames)}
                    if nq == len(qnames) else None)
        quad = {"value": world * 1000.0 / max_over_ranks(q_ms, dist, dev), "unit": "frames/s", "ms_per_step": q_ms,
                "num_keys": num_q, "image_identical_to_tile_keys": same, "stages_ms": q_stages,
                "what": "the same E2E frame through GSR_QUAD_KEYS: one sort key per 2x2 group of 16x16 tiles"}

    # ---- e2e through the public API
    e2e_fps = None
    if not args.quick:
        host = torch.empty((cam.height, cam.width, 3), dtype=torch.uint8, pin_memory=True)
        for _ in range(2):
            img = rast.forward(scene, cam, bg, render_variant=E2E_VARIANT)
            host.copy_(img, non_blocking=True)
        torch.cuda.synchronize()
        Ke = max(5, K // 2)
        t0 = time.perf_counter()
        for _ in range(Ke):
            img = rast.forward(scene, cam, bg, render_variant=E2E_VARIANT)
            host.copy_(img, non_blocking=True)
            torch.cuda.current_stream().synchronize()
        e2e_s = time.perf_counter() - t0
        e2e_fps = world * Ke / e2e_s

    # ---- the reference's own GPU pipeline on this GB300 (its kernels + its CUB sort call)
    ref_gpu = None
    try:
        from oracle import refkernels as RK

        if RK.available() and world == 1 and not args.quick:
            # the reference writes keys unchecked: size its buffers from this
            # library's (capacity-safe) count with a wide margin
            cap_ref = max(1 << 20, 2 * num)
            pipe = RK.Pipeline(scene, cam_spec, cap_ref)
            for _ in range(3):
                pipe.forward()
            torch.cuda.synchronize()
            ts = []
            for _ in range(K):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record()
                n_ref = pipe.forward()
                b.record()
                b.synchronize()
                ts.append(a.elapsed_time(b))
            ref_ms = statistics.mean(ts)
            ref_first = pipe.out.clone()
            pipe.forward()
            torch.cuda.synchronize()
            ds = (pipe.out.int() - ref_first.int()).abs()
            ref_self = {"max_abs": int(ds.max()), "frac_diff": float((ds > 0).double().mean())}
            mine = rast.forward(scene, cam, bg, render_variant=E2E_VARIANT)
            ref_img_equal = bool(torch.equal(pipe.out, mine))
            d = (pipe.out.int() - mine.int()).abs()
            mse = float((d.double() ** 2).mean())
            img_cmp = {"max_abs": int(d.max()), "frac_diff": float((d > 0).double().mean()),
                       "psnr_db": (10.0 * np.log10(255.0 ** 2 / mse)) if mse > 0 else None}
            ref_gpu = {"value": 1000.0 / ref_ms, "unit": "frames/s", "ms_per_frame": ref_ms,
                       "median_ms": statistics.median(ts), "num_rendered": n_ref, "image_identical": ref_img_equal,
                       "image_vs_this_library": img_cmp,
                       "reference_run_vs_run": ref_self,
                       "what": "reference preprocess/render kernels built from its sources + its CUB SortPairs "
                               "call, E2E sequence of forward_fused_e2e incl. its per-frame count read-back"}
            del pipe
            torch.cuda.empty_cache()
    except Exception as exc:  # the comparison is informative, not required
        ref_gpu = {"unavailable": str(exc)[:200]}

    line = None
    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu_baseline and not args.quick:
            cfps, threads, n, el = cpu_frames(raw, cam_spec, seconds=15.0)
            cpu = {"value": cfps, "unit": "frames/s", "cores": threads, "kind": "port",
                   "sample": "%d whole frames of %s in %.1f s (FP64 oracle, %d threads)" % (n, args.workload, el,
                                                                                          threads)}
        if df:
            # counting pass + massive count, compact, depth sort (upsweep + 4),
            # offsets, two emission kernels, tile sort, tile ranges, render
            launches_per_frame = 2 + 1 + 5 + 1 + 2 + 1 + tile_passes + 1 + 1
        else:
            # preprocess + massive emission + upsweep + digit passes + tile ranges + render
            launches_per_frame = 2 + 1 + passes + 1 + 1
        line = {"metric": "frames/s", "value": fps, "unit": "frames/s", "n_gpus": world, "steps": K,
                "warmup": max(3, args.warmup), "ms_per_step": elapsed_ms / K, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": args.workload, "gaussians": P, "width": cam.width, "height": cam.height,
                           "tile": "16x16", "variant": E2E_VARIANT, "sh": "fp16", "num_rendered": num,
                           "pipeline": args.pipeline,
                           "sort_bits": end_bit, "sort_working_passes": len(working), "l2": "inputs larger than L2 (scene %.0f MB)" %
                           (scene.device_bytes() / 1e6), "parallelism": "replicas" if world > 1 else "single"},
                "stages_ms": stage_avg, "quad_keys": quad, "roofline": roofline, "cpu_baseline": cpu,
                "reference_gpu": ref_gpu,
                "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": 60,
                        "d2h_bytes_per_step": cam.width * cam.height * 3 + 4},
                "gpu_launches": launches_per_frame * K, "clocks": clocks}
    return line


def run_serve_profile(args, dev):
    """The served stream alone with a fixed configuration, for profiling."""
    import torch

    from polysplat_gb300 import Scene, scenes
    from polysplat_gb300.serving import Server, TuneConfig

    raws, reqs = scenes.serve_mix()
    scs = [Scene.from_raw(r, dev, keep_fp32_sh=False) for r in raws]
    cfg = TuneConfig(**json.loads(args.serve_profile))
    srv = Server(scs, dev, 60 << 30, cfg)
    for _ in range(2):
        srv.run(reqs, realtime=False, deliver=False)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    st = srv.run(reqs, realtime=False, deliver=False)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    srv.close()
    return {"workload": "serve_mix (profiling run)", "tuned": dataclasses.asdict(cfg), "served": st.as_dict()}


def _img_cmp(a, b):
    """max-abs (in 1/255), differing pixels and PSNR of two uint8 images on the device."""
    import math

    d = (a.int() - b.int()).abs()
    mse = float((d.double() ** 2).mean())
    return int(d.max()), int((d > 0).sum()), (10.0 * math.log10(255.0 ** 2 / mse)) if mse > 0 else float("inf")


def stream_parity(scs, reqs, served, plain, dev):
    """Every request's served image and plain-forward image against the
    reference build's own E2E render of the same request (its preprocess
    and fused render kernels built from its sources, and its CUB sort call,
    on this GPU).  Bar per request: max-abs <= 2/255 and PSNR >= 50 dB."""
    import torch

    from oracle import refkernels as RK

    if not RK.available():
        return {"unavailable": "reference device images not built"}
    cap = max(1 << 20, int(1.25 * max(n for _, n in plain)))
    pipe = RK.Pipeline(max(scs, key=lambda s: s.num_vertex), reqs[0].camera, cap)
    rows = {"served": [], "plain": []}
    for r, img_s, (img_p, n) in zip(reqs, served, plain):
        pipe.set_view(scs[r.scene], r.camera)
        m = pipe.forward()
        if m != n:
            rows.setdefault("key_count_mismatch", []).append((r.camera.id, m, n))
        for name, img in (("served", img_s), ("plain", img_p)):
            rows[name].append((r.camera.id, r.camera.width) + _img_cmp(img, pipe.out))
    del pipe
    torch.cuda.empty_cache()

    def summary(rs):
        fails = [x for x in rs if x[2] > 2 or x[4] < 50.0]
        worst = min(rs, key=lambda x: x[4])
        return {"requests": len(rs), "identical": sum(1 for x in rs if x[2] == 0),
                "fail_bar": len(fails), "worst_max_abs": max(x[2] for x in rs),
                "min_psnr_db": None if worst[4] == float("inf") else round(worst[4], 2),
                "worst_request": {"id": worst[0], "width": worst[1], "max_abs": worst[2], "pixels_differ": worst[3]},
                "failures": [{"id": x[0], "width": x[1], "max_abs": x[2], "pixels_differ": x[3],
                              "psnr_db": round(x[4], 2)} for x in fails[:8]]}

    out = {"served_vs_reference": summary(rows["served"]), "plain_vs_reference": summary(rows["plain"]),
           "bar": "max-abs <= 2/255 and PSNR >= 50 dB per request",
           "reference": "the reference's E2E forward (preprocessCUDA, CUB SortPairs, "
                        "renderCUDA_preranges_smem_persistent_lite_fused, 16x16 tiles), built from its sources"}
    mism = rows.get("key_count_mismatch", [])
    out["key_counts"] = {"requests_equal_to_reference": len(reqs) - len(mism),
                         "largest_difference": max([abs(a - b) for _, a, b in mism], default=0),
                         "examples": mism[:4],
                         "what": "the reference's per-tile key count against this library's on the same request; "
                                 "a difference of a key or two out of millions is one tile on an ellipse's edge"}
    return out


def serve_config(raws, reqs, world):
    """The serve_mix workload's config (shared by both arms of the bench)."""
    return {"workload": "serve_mix", "step": "one saturated pass over the 512-request stream",
            "scenes_gaussians": [r.num for r in raws], "requests": len(reqs), "arrival": "Poisson 240/s",
            "resolutions": ["1280x720", "1920x1080", "2560x1440", "3840x2160"], "budget_gb": 60, "sh": "fp16",
            "tile": "16x16", "render": "preranges_smem_persistent_lite_e2e (exit check every 16 Gaussians)",
            "l2": "scenes of 0.5-10 M Gaussians (68 MB-1.4 GB), larger than L2",
            "parallelism": "replicas" if world > 1 else "single"}


# CPU sample of the serve_mix stream: its first requests, in order
CPU_SAMPLE_REQUESTS = 20


def run_serve(args, dev, rank, world, dist):
    """serve_mix: resident scenes of 0.5/2/5/10 M Gaussians, 512 requests
    arriving by a Poisson process at 240/s, resolutions 720p-2160p, 60 GB
    admission budget.  A step is one saturated pass over the whole stream
    (all 512 requests queued at once), served through Server.run with every
    image delivered to pinned host memory; `value` is frames/s over the K
    timed passes.  The plain per-request forward (the reference's usage of
    Rasterizer.forward) is timed the same way, and both run once more in
    real time for latency.  Every served and plain image of the stream is
    compared with the reference build's own render of the same request."""
    import gc

    import torch

    from polysplat_gb300 import Camera, Rasterizer, Scene, scenes
    from polysplat_gb300.serving import PlainServer, Server, TuneConfig, autotune

    budget = 60 << 30
    raws, reqs = scenes.serve_mix()
    # every served path reads FP16 SH: the scenes keep no FP32 copy
    scs = [Scene.from_raw(r, dev, keep_fp32_sh=False) for r in raws]
    torch.cuda.synchronize()
    K = max(1, args.steps if args.steps is not None else 10)
    W = max(3, args.warmup)
    log = (lambda m: print(m, file=sys.stderr, flush=True)) if rank == 0 else None

    def timed_pass(fn):
        """One pass bracketed by device synchronisation and CUDA events on
        the current stream (the passes run on several streams)."""
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        st = fn()
        torch.cuda.synchronize()
        b.record()
        b.synchronize()
        return st, a.elapsed_time(b) / 1000.0

    # plain per-request forward
    plain = PlainServer(scs, 1 << 28, dev)
    plain.run(reqs[:16], realtime=False)
    p_walls = [timed_pass(lambda: plain.run(reqs, realtime=False)[0])[1] for _ in range(3)]
    p_rt, _ = plain.run(reqs, realtime=True)
    del plain
    gc.collect()
    torch.cuda.empty_cache()

    start = TuneConfig(quad=True, large_keys=1 << 40, max_views=8, massive_area=64, huge_area=4096,
                       max_batch_tiles=1 << 14)
    best, table = autotune(scs, reqs[:128], dev, budget_bytes=budget, log=log, start=start)
    srv = Server(scs, dev, budget, best)
    # warm-up passes over the whole stream: every batch shape's graph is
    # captured and the pinned host pool holds a buffer for every request
    for _ in range(W):
        srv.run(reqs, realtime=False, deliver=True)
        for r in reqs:
            srv.release(r)
    sampler = ClockSampler(dev.index or 0)
    if dist is not None:
        dist.barrier()
    sampler.start()
    time.sleep(0.3)
    walls, last = [], None

    def one():
        st = srv.run(reqs, realtime=False, deliver=True)
        for r in reqs:
            srv.release(r)
        return st

    for _ in range(K):
        last, w = timed_pass(one)
        walls.append(w)
    clocks = sampler.stop()
    s_rt = srv.run(reqs, realtime=True, deliver=True)
    for r in reqs:
        srv.release(r)
    s_dev = srv.run(reqs, realtime=False, deliver=False)
    served_imgs = [r.out for r in reqs]
    srv.close()
    del srv
    gc.collect()
    torch.cuda.empty_cache()

    # parity of the whole stream against the reference build (untimed)
    parity = None
    if not args.quick and world == 1:
        rast = Rasterizer(max(scs, key=lambda s: s.num_vertex), 1 << 28, 1 << 17)
        plain_imgs = []
        for r in reqs:
            img, st = rast.forward(scs[r.scene], Camera.from_spec(r.camera), torch.zeros(3),
                                   render_variant=E2E_VARIANT, return_stats=True)
            plain_imgs.append((img.clone(), int(st["num_rendered"])))
        del rast
        torch.cuda.empty_cache()
        try:
            parity = stream_parity(scs, reqs, served_imgs, plain_imgs, dev)
        except Exception as exc:  # informative; the images are checked by the tests too
            parity = {"unavailable": str(exc)[:200]}
        del plain_imgs
    del served_imgs
    gc.collect()
    torch.cuda.empty_cache()

    # the plain forward of plain_3m_1080p on the same GPU: stage times and the
    # roofline of its dominant kernel
    fargs = argparse.Namespace(**vars(args))
    fargs.workload, fargs.steps, fargs.quick, fargs.no_cpu_baseline = "plain_3m_1080p", 200, False, True
    fwd = forward_line(fargs, dev, rank, world, dist)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = serve_cpu_baseline(raws, reqs[:CPU_SAMPLE_REQUESTS], seconds=60.0)
    total = max_over_ranks(sum(walls), dist, dev)
    value = world * K * len(reqs) / total
    per_pass = sorted(len(reqs) / w for w in walls)
    p_fps = sorted(len(reqs) / w for w in p_walls)
    img_bytes = sum(r.camera.width * r.camera.height * 3 for r in reqs)
    # kernel launches of one saturated pass: small batches (preprocess,
    # large-Gaussian emission, upsweep, 6 digit passes, ranges, render) and
    # large frames (20 launches of the depth-first forward)
    launches = K * (last.batches * 11 + last.large * 20)
    if rank != 0:
        return None
    med = statistics.median
    return {"metric": "frames/s", "value": value, "unit": "frames/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": 1000.0 * total / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": serve_config(raws, reqs, world),
            "gpu_launches": launches, "clocks": clocks, "cpu_baseline": cpu,
            "roofline": dict(fwd["roofline"], workload="plain_3m_1080p (plain forward)") if fwd else None,
            "forward": {k: fwd[k] for k in ("value", "ms_per_step", "stages_ms", "quad_keys", "e2e", "reference_gpu",
                                            "config")} if fwd else None,
            "autotune": {"candidates": len(table), "sample_requests": 128,
                         "best_sample_frames_per_s": max(f for _, f in table)},
            "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 376 * len(reqs),
                    "d2h_bytes_per_step": int(img_bytes)},
            "served": {"tuned": dataclasses.asdict(best),
                       "saturated_frames_per_s": {"median": med(per_pass), "min": per_pass[0], "max": per_pass[-1],
                                                  "passes": K},
                       "device_only_frames_per_s": s_dev.frames_per_s, "batches_per_pass": last.batches,
                       "large_lane_per_pass": last.large, "retries": last.retries, "failed": last.failed,
                       "realtime_240hz": {"p50_ms": s_rt.p50_ms, "p99_ms": s_rt.p99_ms,
                                          "p99_1080p_ms": s_rt.p99_1080p_ms, "frames_per_s": s_rt.frames_per_s}},
            "plain": {"saturated_frames_per_s": {"median": med(p_fps), "min": p_fps[0], "max": p_fps[-1],
                                                 "passes": len(p_fps)},
                      "realtime_240hz": {"p50_ms": p_rt.p50_ms, "p99_ms": p_rt.p99_ms,
                                         "p99_1080p_ms": p_rt.p99_1080p_ms}},
            "parity_vs_reference": parity,
            "headline": {"served_frames_per_s": value, "plain_frames_per_s": med(p_fps),
                         "speedup_vs_plain": value / med(p_fps), "served_p99_1080p_ms": s_rt.p99_1080p_ms,
                         "served_p99_ms": s_rt.p99_ms, "plain_p99_ms": p_rt.p99_ms,
                         "served_min_psnr_vs_reference_db": (parity or {}).get("served_vs_reference", {}).get(
                             "min_psnr_db"),
                         "served_requests_failing_bar": (parity or {}).get("served_vs_reference", {}).get(
                             "fail_bar")}}


def _timed_launches(fn, K, warmup, dev, dist):
    """Average ms of `fn` over K back-to-back calls (CUDA events on the current
    stream, max over ranks), with the SM clocks sampled meanwhile."""
    import torch

    for _ in range(max(3, warmup)):
        fn()
    sampler = ClockSampler(dev.index or 0)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    stream = torch.cuda.current_stream(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(K):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    return max_over_ranks(a.elapsed_time(b) / K, dist, dev), clocks


def run_gather(args, dev, rank, world, dist):
    """The feature gather (gather_features; the reference's gather.cu:6-22)
    alone, over the sorted values of one plain_3m_1080p frame: per key, the
    4-byte index, a random read of the Gaussian's 40 bytes of features
    (xy, rgb + depth, conic + log2 opacity) and a sequential 40-byte write.
    `value` is GB/s of those algorithmic bytes, CUDA-event timed; the 9.2 M
    keys move 773 MB per step, larger than L2."""
    import torch

    from polysplat_gb300 import Camera, Rasterizer, Scene, ops, scenes

    raw, cams = scenes.workload("plain_3m_1080p")
    scene = Scene.from_raw(raw, dev)
    cam = Camera.from_spec(cams[0])
    cap = 1 << 26
    rast = Rasterizer(scene, cap, 1 << 18)
    rast.forward(scene, cam, torch.zeros(3), render_variant="preranges_smem_persistent_lite_e2e", use_es=False)
    torch.cuda.synchronize()
    M = int(rast.curr_offset.item())
    vals = rast.gaussian_values_sorted[:M]
    dst = [torch.empty((M, k), device=dev, dtype=torch.float32) for k in (2, 4, 4)]
    src = (rast.points_xy, rast.rgb_depth, rast.conic_opacity)
    per_key = 4 + 2 * sum(t.shape[1] * 4 for t in dst)
    K = max(3, args.steps)
    ms, clocks = _timed_launches(lambda: ops.gather_features(M, vals, *src, *dst), K, args.warmup, dev, dist)
    if rank != 0:
        return None
    gbs = world * M * per_key / (ms * 1e-3) / 1e9
    peak = measured_peaks()
    return {"metric": "GB/s", "value": gbs, "unit": "GB/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "gather_plain_3m_1080p", "keys": M, "bytes_per_key": per_key,
                       "l2": "%.0f MB per step, larger than L2; the %.0f MB feature table it reads at random can "
                             "stay in L2" % (M * per_key / 1e6, sum(t.numel() * 4 for t in src) / 1e6),
                       "parallelism": "single"},
            "roofline": {"bound": "hbm", "kernel": "k_gather", "achieved": gbs / world, "peak": peak[0],
                         "unit": "GB/s", "frac": gbs / world / peak[0], "peak_kind": peak[1], "traffic": None},
            "gpu_launches": K, "clocks": clocks}


def run_prepare(args, dev, rank, world, dist):
    """The scene transform (gsr_scene_prepare; the reference's CPU loop in
    loadPly_torch / computeCov3D, pybind.cpp:22-56, 105-117) alone on the
    3 M Gaussians of plain_3m_1080p: per Gaussian it reads log-scales,
    quaternion and opacity logit (32 B) and writes opacity and the 3D
    covariance (28 B).  `value` is GB/s of those 60 bytes per Gaussian."""
    import torch

    from polysplat_gb300 import scenes
    from polysplat_gb300._lib import check, lib

    raw, _ = scenes.workload("plain_3m_1080p")
    P = raw.num
    t = lambda a: torch.from_numpy(a.reshape(P, -1)).to(dev).contiguous()
    ls, q, lg = t(raw.log_scales), t(raw.quats), t(raw.opacity_logits)
    op = torch.empty(P, dtype=torch.float32, device=dev)
    cov = torch.empty((P, 6), dtype=torch.float32, device=dev)
    L = lib()
    sh = torch.cuda.current_stream(dev).cuda_stream

    def launch():
        check(L.gsr_scene_prepare(P, ls.data_ptr(), q.data_ptr(), lg.data_ptr(), op.data_ptr(), cov.data_ptr(), sh),
              "scene_prepare")

    K = max(3, args.steps)
    ms, clocks = _timed_launches(launch, K, args.warmup, dev, dist)
    if rank != 0:
        return None
    per = 32 + 28
    gbs = world * P * per / (ms * 1e-3) / 1e9
    peak = measured_peaks()
    return {"metric": "GB/s", "value": gbs, "unit": "GB/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "prepare_plain_3m", "gaussians": P, "bytes_per_gaussian": per,
                       "l2": "%.0f MB per step, %.1fx L2: part of it can stay in L2 between launches"
                             % (P * per / 1e6, P * per / 129e6), "parallelism": "single"},
            "roofline": {"bound": "hbm", "kernel": "k_scene_prepare", "achieved": gbs / world, "peak": peak[0],
                         "unit": "GB/s", "frac": gbs / world / peak[0], "peak_kind": peak[1], "traffic": None},
            "gpu_launches": K, "clocks": clocks}


def run_diff(args, dev, rank, world, dist):
    """diff_1m_8cam: 1 M Gaussians (means ~ N(0, 3^2 I)), 8 cameras at 1280x720 on
    a radius-10 orbit, L2 loss against renders of perturbed means and SH DC.
    A step is the forward of the 8 views, the loss and the backward to every
    raw parameter; `value` is views per second through `render_views` (all
    views in one pass, quad keys), `one_pass_per_tile_keys` the same with
    per-tile keys, and `per_view_passes` the same step with one forward and
    backward per camera."""
    import numpy as np
    import torch

    from polysplat_gb300 import Camera, scenes
    from polysplat_gb300.diff import render, render_views

    raw, cams = scenes.workload("diff_1m_8cam")
    rng = np.random.default_rng(4)
    cams = [Camera.from_spec(c) for c in cams]
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device=dev)
    params = [t(raw.means), t(raw.log_scales), t(raw.quats), t(raw.opacity_logits), t(raw.shs.reshape(-1, 48))]
    tm = t(raw.means + rng.normal(0, 0.05, raw.means.shape))
    tsh = raw.shs.copy()
    tsh[:, 0, :] += rng.normal(0, 0.1, tsh[:, 0, :].shape)
    with torch.no_grad():
        targets = [render(tm, params[1], params[2], params[3], t(tsh.reshape(-1, 48)), c) for c in cams]
    for p in params:
        p.requires_grad_(True)

    tstack = torch.stack(targets)

    def step(multi=True, quad=True):
        for p in params:
            p.grad = None
        if multi:
            # all views as one [views, H, W, 3] tensor: the L2 loss is one operation
            loss = ((render_views(*params, cams, quad_keys=quad, stacked=True) - tstack) ** 2).sum()
        else:
            loss = sum(((render(*params, c) - tg) ** 2).sum() for c, tg in zip(cams, targets))
        loss.backward()
        return loss

    K = max(3, min(args.steps, 30))
    if args.diff_profile:
        for multi, name in ((True, "timed_views"), (False, "timed_loop")):
            for _ in range(3):
                step(multi)
            torch.cuda.synchronize()
            # a start/end range, not push/pop: the backward launches from
            # autograd's own thread
            rid = torch.cuda.nvtx.range_start(name)
            step(multi)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_end(rid)
        return {"workload": "diff_1m_8cam (profiling run)", "ranges": ["timed_views", "timed_loop"]}

    def timed(multi, sampler=None, quad=True):
        for _ in range(max(3, args.warmup)):
            step(multi, quad)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        if sampler is not None:
            sampler.start()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(K):
            step(multi, quad)
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / K

    sampler = ClockSampler(dev.index or 0)
    ms = timed(True, sampler)
    clocks = sampler.stop()
    ms_loop = timed(False)
    ms_tile = timed(True, quad=False)
    ms = max_over_ranks(ms, dist, dev)
    ms_loop = max_over_ranks(ms_loop, dist, dev)
    ms_tile = max_over_ranks(ms_tile, dist, dev)
    if rank != 0:
        return None
    views = world * len(cams) * 1000.0 / ms
    # library kernels per step: scene transform, preprocess and large-Gaussian
    # emission, sort upsweep and digit passes, tile ranges, render, render
    # backward, one adjoint per 16 views
    quads = ((1280 // 16 + 1) // 2) * (((720 + 15) // 16 + 1) // 2) * len(cams)
    sort_passes = (32 + int(quads).bit_length() + 7) // 8
    launches = 1 + 2 + 1 + sort_passes + 1 + 1 + 1 + (len(cams) + 15) // 16
    return {"metric": "views/s (forward + backward)", "value": views, "unit": "views/s", "n_gpus": world,
            "steps": K, "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "diff_1m_8cam", "gaussians": raw.num, "views": len(cams),
                       "resolution": "1280x720", "loss": "L2", "grads": "means, log-scales, quats, logits, SH",
                       "l2": "scene 1 M Gaussians (0.3 GB fp32 parameters + per-view lists), larger than L2"},
            "per_view_passes": {"value": world * len(cams) * 1000.0 / ms_loop, "unit": "views/s",
                                "ms_per_step": ms_loop},
            "one_pass_per_tile_keys": {"value": world * len(cams) * 1000.0 / ms_tile, "unit": "views/s",
                                       "ms_per_step": ms_tile},
            "e2e": {"value": views, "unit": "views/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 4},
            "gpu_launches": K * launches, "clocks": clocks}


def serve_cpu_baseline(raws, reqs, seconds: float):
    """The FP64 oracle on the host cores, rendering the request stream in
    order for about `seconds` (at least one request)."""
    from oracle import oracle as O
    from polysplat_gb300.rasterizer import Camera

    threads = O.nthreads_default()
    prepared = {}
    n, t0 = 0, time.perf_counter()
    for r in reqs:
        if r.scene not in prepared:
            raw = raws[r.scene]
            prepared[r.scene] = O.scene_transform(raw.log_scales, raw.quats, raw.opacity_logits)
        op, cov = prepared[r.scene]
        raw = raws[r.scene]
        O.forward(raw.means, raw.shs, op, cov, r.camera, cadence=16, half_sh=True, nthreads=threads)
        n += 1
        if time.perf_counter() - t0 > seconds:
            break
    el = time.perf_counter() - t0
    return {"value": n / el, "unit": "frames/s", "cores": threads, "kind": "port", "requests": n, "seconds": el,
            "sample": "the first %d requests of the serve_mix stream in %.1f s (FP64 oracle, %d threads; scene "
                      "transforms included)" % (n, el, threads)}


def run_reference_gpu(args):
    """The reference's own GPU pipeline alone (its kernels + its CUB sort call),
    for timing and kernel-level profiling next to this library."""
    import torch

    from oracle import refkernels as RK
    from polysplat_gb300 import Camera, Rasterizer, Scene, scenes

    if not RK.available():
        print(json.dumps({"impl": "reference-gpu", "unavailable": "reference device images not built"}))
        return 0
    dev = torch.device("cuda", 0)
    raw, cams = scenes.workload(args.workload)
    scene = Scene.from_raw(raw, dev)
    spec = cams[0]
    # count the keys with this library first (its writes are clamped); the
    # reference writes unchecked, so its buffers get a wide margin
    probe = Rasterizer(scene, 1 << (args.cap_log2 or 26), 1 << 18)
    _, st = probe.forward(scene, Camera.from_spec(spec), torch.zeros(3), render_variant=E2E_VARIANT,
                          return_stats=True)
    del probe
    torch.cuda.empty_cache()
    pipe = RK.Pipeline(scene, spec, max(1 << 20, 2 * st["num_rendered"]))
    for _ in range(max(3, args.warmup)):
        pipe.forward()
    torch.cuda.synchronize()
    ts = []
    for _ in range(args.steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        n = pipe.forward()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    ms = statistics.mean(ts)
    print(json.dumps({"impl": "reference-gpu", "metric": "frames/s", "value": 1000.0 / ms, "unit": "frames/s",
                      "ms_per_step": ms, "steps": args.steps, "num_rendered": n,
                      "config": {"workload": args.workload}}), flush=True)
    return 0


def main():
    args = parse()
    if args.steps is None and args.workload != "serve_mix":
        args.steps = 500
    if args.impl == "reference":
        return run_reference(args)
    if args.impl == "reference-gpu":
        return run_reference_gpu(args)
    return run_gsr(args)


if __name__ == "__main__":
    sys.exit(main())
