"""Benchmark of the sofren2 per-frame render path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config 2]

A step is one frame of the workload: the frame's API calls (lights, camera, instances with
posed bones) and sft_present through the library, i.e. proxy occlusion, geometry, binning,
tile raster and resolve on the GPU.  The default workload is the skinned-characters scene
(eight ~6k-triangle humanoids on a 22-joint skeleton, ground of 64x64 quads, four point
lights, 512x512 textures) at 1920x1080 with 2x MSAA; `--config 1|3` selects the static
640x360 scene or the 262k-triangle lightmapped atrium at 1920x1080 with 4x MSAA; `--config 4|5`
the batched multi-view and served workloads; `--config 6` ray queries (2^20 rays against the
atrium scene, rays/s); `--config 7` the BLAS build of the 249k-triangle atrium model at model
creation (triangles/s); `--config 8` skeletal poses (2^16 requests on a 22-bone rig, poses/s).

  value   frames/s with the scene resident in device memory and the colour left there
  e2e     frames/s through the public API into a host colour buffer (pinned staging of the
          frame inputs H2D, the 1080p colour buffer D2H, every step)

Timing: W untimed warm-up steps, then K steps each bracketed by CUDA events on the library's
stream with an L2 flush (a 512 MiB device write) between steps, outside the events.  Under
torchrun each rank renders its own frames on its own GPU (replicas, weak scaling); the job
time is the max over ranks.  `--impl reference` times the reference's own render path
(sofren2.c unmodified, built on this host by `make -C oracle ref_bench`: its NEON path on an
aarch64 host, AVX2 on x86-64) with its own worker pool on all host cores, over a bounded sample
of frames; where that build is absent, the CPU restatement of the reference algorithm
(oracle/sft_oracle.c), and the line says which (`cpu_baseline.kind`).  The same two CPU legs,
reference first, form the `cpu_baseline` of the frame workloads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

CONFIGS = {
    1: dict(gen="config1", samples=1, name="static_640x360_1x", width=640, height=360),
    2: dict(gen="config2", samples=2, name="skinned_1080p_2xmsaa", width=1920, height=1080),
    3: dict(gen="config3", samples=4, name="atrium_1080p_4xmsaa", width=1920, height=1080),
    4: dict(gen="config4", samples=None, name="multiview_96_views_6_scenes", width=None, height=None),
    5: dict(gen="config5", samples=None, name="served_16_scenes_poisson", width=None, height=None),
    6: dict(gen="config3", samples=None, name="raycast_atrium_1m_rays", width=None, height=None, rays=1 << 20),
    7: dict(gen="config3", samples=None, name="blas_build_atrium_249k_triangles", width=None, height=None, model=0),
    8: dict(gen=None, samples=None, name="pose_22_bones_65536_requests", width=None, height=None, requests=1 << 16),
}
SERVE_RATES = (100, 500, 1000, 1500, 2000, 5000)   # requests/s offered
SERVE_BUDGET = 150 << 30                      # device-memory admission budget, bytes


def max_over_ranks(values: list[float], device: str = "cpu") -> list[float]:
    """Element-wise max of per-rank timings over the process group (identity without one): the
    job's time is its slowest rank's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(values)
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_throughput(units_per_rank: int, world: int, ms_max: float) -> float:
    """Whole-job rate: the units every rank processed over the slowest rank's time."""
    return units_per_rank * world / (ms_max * 1e-3)


def _peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": float(d["hbm_gbs"]), "src": "measured", "sm_max_mhz": float(d.get("sm_max_mhz", 2070.0))}
    return {"hbm_gbs": 6800.0, "src": "fallback", "sm_max_mhz": 2070.0}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc, self.lines = index, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0])); mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# The resolve phase of one frame of the workload (k_resolve, and k_tile_lights where the range makes
# its light lists once per tile), from full ncu captures on a GB300 (`-k regex:"k_resolve|k_tile_lights"`
# on `bench.py --steps 2 --warmup 3 --config N --no-cpu-baseline`, summarised in
# profiles/k_resolve_*.md, same kernel code as the library's): DRAM bytes (dram__bytes_read.sum +
# dram__bytes_write.sum), warp instructions issued (smsp__inst_executed.sum), and the issue-active
# and FMA-pipe fractions ncu measured over the kernel's active cycles.
RESOLVE_PROFILE = {
    "skinned_1080p_2xmsaa": {"traffic": 38166528 + 65792, "instructions": 150347274, "issue_active": 0.599, "fma_pipe": 0.223,
                             "profile": "profiles/k_resolve_skinned_1080p_2x.md"},
    # the resolve phase here is k_tile_lights (1528470 instructions, no DRAM traffic to speak of) then k_resolve<4>
    "atrium_1080p_4xmsaa": {"traffic": 75378432 + 3088384 + 36352, "instructions": 360592456 + 1528470, "issue_active": 0.588,
                            "fma_pipe": 0.204, "profile": "profiles/k_resolve_atrium_1080p_4x.md"},
    "static_640x360_1x": {"traffic": 2486528, "instructions": 5135702, "issue_active": 0.312, "fma_pipe": 0.072,
                          "profile": "profiles/k_resolve_static_640x360_1x.md"},
}


def resolve_roofline(name: str, W: int, H: int, S: int, tile_ms: float, clk: dict, peaks: dict) -> dict:
    """k_resolve is issue bound (FP32 shading of lights x capsule proxies per pixel, DRAM a few %):
    the roofline is its issue rate, warp instructions per launch (ncu) over the live CUDA-event
    time, against 4 schedulers per SM at the SM clock sampled during the run.  The HBM form of
    the contract (algorithmic bytes over time against the measured copy bandwidth) rides along."""
    import torch
    alg = _algorithmic_resolve_bytes(W, H, S)
    gbs = alg / (tile_ms * 1e-3) / 1e9 if tile_ms > 0 else 0.0
    prof = RESOLVE_PROFILE.get(name)
    hbm = {"achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": gbs / peaks["hbm_gbs"],
           "traffic": prof["traffic"] if prof else None, "algorithmic_bytes": alg, "peak_source": peaks["src"]}
    if not prof or tile_ms <= 0:
        return {"kernel": "k_resolve", "bound": "hbm", **hbm, "note": "no ncu instruction count for this workload"}
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = float(clk.get("sm_mhz") or peaks.get("sm_max_mhz") or 2070.0)
    peak = sms * 4 * mhz * 1e6
    ach = prof["instructions"] / (tile_ms * 1e-3)
    return {"kernel": "k_resolve", "bound": "issue", "achieved": ach, "peak": peak, "unit": "warp-instructions/s",
            "frac": ach / peak, "traffic": prof["traffic"], "instructions_per_launch": prof["instructions"],
            "peak_from": f"{sms} SMs x 4 schedulers x {mhz:.0f} MHz (median SM clock sampled in the run)",
            "ncu": {"issue_active": prof["issue_active"], "fma_pipe": prof["fma_pipe"], "source": prof["profile"]}, "hbm": hbm}


def _algorithmic_resolve_bytes(width: int, height: int, samples: int) -> float:
    """Bytes the resolve kernel must move per frame at minimum: per pixel the visibility
    buffer (8 B per sample: depth and id), the vertex data of its triangle (156 B per distinct
    triangle of a 4x2 block, about one per block, so 156/8 B per pixel), 4 bilinear texels
    (16 B) and the colour write (4 B)."""
    pixels = width * height
    return pixels * (8.0 * samples + 156.0 / 8 + 16 + 4)


def run_ours(args, cfg) -> dict:
    import torch
    import torch.distributed as dist
    from sofren2_gb300 import runtime, scenes

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    os.environ["SFT_CUDA_DEVICE"] = str(local)
    sc = getattr(scenes, cfg["gen"])()
    blob = sc.to_bytes()
    W, H, S = cfg["width"], cfg["height"], cfg["samples"]
    R = runtime.Renderer(W, H, S)
    h = R.load_scene(blob)
    stream = torch.cuda.ExternalStream(R.stream(), device=torch.device("cuda", local))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    color = np.zeros((H, W), dtype=np.uint32)
    # pin the host colour buffer like a swapchain staging buffer
    color_t = torch.from_numpy(color).pin_memory() if torch.cuda.is_available() else None
    color = color_t.numpy() if color_t is not None else color

    def device_step():
        R.render_device(h, 0)

    def e2e_step():
        R.render(h, 0, color)

    def timed(step, n, kern=None):
        """n steps, each bracketed by CUDA events on the renderer's stream; kern (optional)
        accumulates the library's per-phase event timings of every timed step."""
        times = []
        for _ in range(n):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            if kern is not None:
                kern += R.timings()
        return times

    for _ in range(args.warmup):
        device_step()
        e2e_step()
    tss, npx = runtime.scene_counts(sc)
    dbg = R.render_debug(h, 0, tss, npx, payload_cap=1 << 24)
    payloads = int(dbg["tile_payloads"].size)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    kern = np.zeros(5)
    dev_times = timed(device_step, args.steps, kern)
    launches = R.launch_count() * args.steps
    kern /= args.steps
    e2e_times = timed(e2e_step, args.steps)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    ms_dev = float(np.sum(dev_times))
    ms_e2e = float(np.sum(e2e_times))
    ms_dev, ms_e2e = max_over_ranks([ms_dev, ms_e2e], device=f"cuda:{local}")
    frames = args.steps * world
    peaks = _peaks()
    tile_ms = float(kern[4])
    h2d = 4096 + sum(16 * 4 * (len(b) if b is not None else 0) for _, _, b in sc.frames[0].instances)
    line = {
        "metric": "frames_per_second", "value": job_throughput(args.steps, world, ms_dev), "unit": "frames/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scene)",
        "config": frame_config(cfg),
        "workload_detail": {"global_batch": world,
                            "triangles": int(sum(int((ms.inds.reshape(-1, 16, 32)[:, :, :24].reshape(-1, 16, 3, 8)).any(axis=2).sum())
                                                 for mi, _, _ in sc.frames[0].instances for ms in sc.models[mi].meshes)),
                            "l2": "flushed between steps (512 MiB device write, outside the timed events)",
                            "parallelism": f"replicas x{world}"},
        "e2e": {"value": job_throughput(args.steps, world, ms_e2e), "unit": "frames/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(W * H * 4)},
        "gpu_launches": int(launches),
        "kernel_ms": {"occlusion": float(kern[0]), "geometry": float(kern[1]), "binning": float(kern[2]),
                      "raster": float(kern[3]), "resolve": tile_ms},
        "roofline": resolve_roofline(cfg["name"], W, H, S, tile_ms, clk, peaks),
        "clocks": clk,
        "wall_s": wall,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(blob, S, W, H, seconds=args.cpu_seconds)
    R.free_scene(h)
    R.close()
    if world > 1:
        dist.destroy_process_group()
    return line if rank == 0 else None


def run_batch(args, cfg) -> dict:
    """Config 4: all views rendered as one batched submission per step (sftg_frames_render)
    against the plain path (one sft_present per view) on the same GPU, both after the
    autotuner picked the scheduling knobs on this view set."""
    import torch
    import torch.distributed as dist
    from sofren2_gb300 import runtime, scenes

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    os.environ["SFT_CUDA_DEVICE"] = str(local)
    scs, vlist = scenes.config4()
    blobs = [sc.to_bytes() for sc in scs]
    R = runtime.Renderer(640, 360, 1)
    hs = [R.load_scene(b) for b in blobs]
    views = [(hs[si], f, S) for si, f, S in vlist]
    sizes = [(scs[si].frames[f].width, scs[si].frames[f].height, S) for si, f, S in vlist]
    stream = torch.cuda.ExternalStream(R.stream(), device=torch.device("cuda", local))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    pinned = [torch.zeros((h, w), dtype=torch.int32).pin_memory() for w, h, _ in sizes]   # kept alive with the views
    colors = [t.numpy().view(np.uint32) for t in pinned]

    lanes = [0]   # 0: one submission; k >= 1: k submissions overlapping on lanes 1..k (picked below)

    def batched_device():
        R.render_batch(views, None, lanes=lanes[0])

    def batched_e2e():
        R.render_batch(views, colors, lanes=lanes[0])

    single_tuning = R.tuning()   # the knobs measured best on single views (the context's defaults)

    def plain_device():   # each view with the single-view knobs, restored after
        R.set_tuning(**single_tuning)
        for h, f, S in views:
            R.set_samples(S)
            R.render_device(h, f)
        R.set_tuning(**tuning)

    def timed(step, n, kern=None):
        times = []
        for _ in range(n):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            if kern is not None:
                kern += R.timings()
        return times

    tuning = R.autotune_batch(views, reps=3)   # the knobs for the batch; the plain path keeps single_tuning
    lane_ms = {}
    for k in (0, 2, 3, 4):   # the submission split: whole batch, or 2-4 overlapping batches
        lanes[0] = k
        for _ in range(2):
            batched_device()
        lane_ms[k] = float(np.median(timed(batched_device, 3)))
    lanes[0] = min(lane_ms, key=lane_ms.get)
    for _ in range(args.warmup):
        batched_device()
        batched_e2e()
        plain_device()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    kern = np.zeros(5)
    if lanes[0]:   # phase timings and launch count of the same views as one submission (one set of kernels)
        chosen = lanes[0]
        lanes[0] = 0
        timed(batched_device, args.steps, kern)
        launches = R.launch_count() * args.steps
        lanes[0] = chosen
        l0 = R.launch_total()
        dev = timed(batched_device, args.steps)
        launches = R.launch_total() - l0
    else:
        dev = timed(batched_device, args.steps, kern)
        launches = R.launch_count() * args.steps
    kern /= args.steps
    e2e = timed(batched_e2e, args.steps)
    plain = timed(plain_device, args.steps)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    ms_dev, ms_e2e, ms_plain = float(np.sum(dev)), float(np.sum(e2e)), float(np.sum(plain))
    ms_dev, ms_e2e, ms_plain = max_over_ranks([ms_dev, ms_e2e, ms_plain], device=f"cuda:{local}")
    n = len(views)
    frames = n * args.steps * world
    peaks = _peaks()
    alg = sum(_algorithmic_resolve_bytes(w, h, S) for w, h, S in sizes)
    achieved = alg / (kern[4] * 1e-3) / 1e9 if kern[4] > 0 else 0.0
    h2d = sum(4096 + sum(16 * 4 * (len(b) if b is not None else 0) for _, _, b in scs[si].frames[f].instances)
              for si, f, _ in vlist)
    msaa = {str(k): sum(1 for _, _, S in sizes if S == k) for k in (1, 2, 4)}
    line = {
        "metric": "frames_per_second", "value": frames / (ms_dev * 1e-3), "unit": "frames/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scenes, seeded cameras)",
        "config": {"workload": cfg["name"], "views": n, "scenes": len(scs), "global_batch": n * world,
                   "resolutions": sorted({f"{w}x{h}" for w, h, _ in sizes}), "views_per_msaa": msaa,
                   "megapixels_per_step": round(sum(w * h for w, h, _ in sizes) / 1e6, 2),
                   "l2": "flushed between steps (512 MiB device write, outside the timed events)",
                   "parallelism": f"replicas x{world}", "tuning": tuning,
                   "submission": ("one batch" if lanes[0] == 0 else f"{lanes[0]} batches overlapping on submission lanes"),
                   "submission_ms": {("one batch" if k == 0 else f"{k} lanes"): round(v, 3) for k, v in lane_ms.items()}},
        "plain": {"value": frames / (ms_plain * 1e-3), "unit": "frames/s", "tuning": single_tuning,
                  "note": "the same views, one sft_present each (one launch sequence per view), with the knobs "
                          "measured best on single views; the batch uses the autotuned knobs"},
        "batched_over_plain": ms_plain / ms_dev,
        "e2e": {"value": frames / (ms_e2e * 1e-3), "unit": "frames/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(sum(w * h * 4 for w, h, _ in sizes))},
        "gpu_launches": int(launches),
        "kernel_ms": {"occlusion": float(kern[0]), "geometry": float(kern[1]), "binning": float(kern[2]),
                      "raster": float(kern[3]), "resolve": float(kern[4])},
        "roofline": {"kernel": "k_resolve", "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": None, "peak_source": peaks["src"],
                     "note": "the resolve is FP32/issue bound; HBM fraction of its algorithmic bytes shown per contract"},
        "clocks": clk,
        "wall_s": wall,
    }
    if rank == 0 and not args.no_cpu_baseline:
        # bounded sample: the first view of every scene, at its own size and MSAA
        fps, kinds = [], set()
        for si in range(len(scs)):
            k = next(i for i, v in enumerate(vlist) if v[0] == si)
            w, h, S = sizes[k]
            cb = cpu_baseline(blobs[si], S, w, h, seconds=args.cpu_seconds / len(scs), frame=vlist[k][1])
            fps.append(cb["value"])
            kinds.add(cb["kind"])
        kind = "reference" if kinds == {"reference"} else "port"
        line["cpu_baseline"] = {"value": len(fps) / sum(1.0 / f for f in fps), "unit": "frames/s", "cores": cb["cores"],
                                "kind": kind, "sample": f"one view of each of the {len(scs)} scenes at its own size and "
                                "MSAA, ~%.0f s each (%s); harmonic mean" % (
                                    args.cpu_seconds / len(scs),
                                    cb["sample"].split(": ", 1)[-1] if kind == "reference" else "oracle/sft_oracle.c, tile-parallel")}
    for h in hs:
        R.free_scene(h)
    R.close()
    if world > 1:
        dist.destroy_process_group()
    return line if rank == 0 else None


def run_serve(args, cfg) -> dict:
    """Config 5: Poisson request streams at several rates over 16 resident scenes, served by the
    native continuous-batching loop (sftx_serve: batches overlapping on the GPU over submission
    lanes), by the same loop with one batch at a time, and by the plain per-request path."""
    import torch
    from sofren2_gb300 import runtime, scenes

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    os.environ["SFT_CUDA_DEVICE"] = str(local)
    scs, samples = scenes.config5()
    R = runtime.Renderer(640, 360, 1)
    hs = [R.load_scene(sc.to_bytes()) for sc in scs]
    meshlets = [[sum(sum(ms.n for ms in sc.models[mi].meshes) for mi, _, _ in fr.instances) for fr in sc.frames] for sc in scs]
    max_batch = 64
    big = max(fr.width * fr.height for sc in scs for fr in sc.frames)
    pinned = [torch.zeros(big, dtype=torch.int32).pin_memory() for _ in range(2 * max_batch)]   # requests in flight
    colors = [t.numpy().view(np.uint32) for t in pinned]

    def make_requests(rate, seconds, seed):
        rng = np.random.default_rng(seed)
        t, out = 0.0, []
        while True:
            t += rng.exponential(1.0 / rate)
            if t > seconds:
                return out
            si = int(rng.integers(len(scs)))
            f = int(rng.integers(len(scs[si].frames)))
            fr = scs[si].frames[f]
            out.append((t, si, f, samples[si], int(rng.integers(1, 17)),
                        runtime.request_device_bytes(fr.width, fr.height, samples[si], meshlets[si][f])))

    def stats(reqs, done, st):
        arr = np.array([r[0] for r in reqs])
        lat = (done - arr) * 1e3
        span = float(done.max() - arr.min())
        hd = np.array([scs[r[1]].frames[r[2]].width == 1920 and scs[r[1]].frames[r[2]].height == 1080 for r in reqs])
        return {"requests": len(reqs), "p50_ms": float(np.percentile(lat, 50)), "p95_ms": float(np.percentile(lat, 95)),
                "p99_ms": float(np.percentile(lat, 99)), "frames_per_second": len(reqs) / span,
                "p99_1080p_ms": float(np.percentile(lat[hd], 99)) if hd.any() else None, "requests_1080p": int(hd.sum()),
                "batches": int(st["batches"]), "mean_batch": len(reqs) / max(1, int(st["batches"])),
                "max_batch": int(st["max_batch"]), "max_batches_in_flight": int(st.get("max_inflight", 1)) or 1,
                "peak_admitted_gb": st["peak_bytes"] / 2**30}

    # warm-up: grow every lane's buffers to the largest batch the runs can form (a lane growing
    # while requests are timed stalls its batch), then run each mode over a short burst
    warm = make_requests(max(SERVE_RATES), 0.05, 1)
    warm = [(0.0,) + r[1:] for r in warm[:max_batch]]
    R.serve_warm(hs, [r for rate in SERVE_RATES for r in make_requests(rate, 1.0, 7)], max_batch, SERVE_BUDGET, colors)
    for _ in range(args.warmup):
        R.serve(hs, warm, max_batch, SERVE_BUDGET, "overlap", colors)
        R.serve(hs, warm, max_batch, SERVE_BUDGET, "batched", colors)
        R.serve(hs, warm[:4], max_batch, SERVE_BUDGET, "plain", colors)
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    points = []
    for k, rate in enumerate(SERVE_RATES):
        reqs = make_requests(rate, args.serve_seconds, 100 + k)
        done, _, st = R.serve(hs, reqs, max_batch, SERVE_BUDGET, "overlap", colors)
        served = stats(reqs, done, st)
        done, _, st = R.serve(hs, reqs, max_batch, SERVE_BUDGET, "batched", colors)
        one_at_a_time = stats(reqs, done, st)
        # the plain path cannot keep up with high rates; offer it at most ~1 s of requests
        preqs = [r for r in reqs if r[0] <= min(args.serve_seconds, 1.0)]
        done, _, st = R.serve(hs, preqs, max_batch, SERVE_BUDGET, "plain", colors)
        points.append({"rate": rate, "batched": served, "batched_one_at_a_time": one_at_a_time, "plain": stats(preqs, done, st)})
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    top = points[-1]["batched"]
    # latency headline: the highest offered rate the serving loop sustains (served at >= 99 % of the
    # offered rate over the run, so that its queue does not grow)
    kept = [p for p in points if p["batched"]["frames_per_second"] >= 0.99 * p["rate"]] or points[:1]
    sla = kept[-1]
    line = {
        "metric": "frames_per_second", "value": top["frames_per_second"], "unit": "frames/s", "n_gpus": 1,
        "steps": len(SERVE_RATES), "warmup": args.warmup, "ms_per_step": 1e3 / top["frames_per_second"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scenes, seeded cameras, Poisson arrivals)",
        "config": {"workload": cfg["name"], "scenes": len(scs), "rates_per_s": list(SERVE_RATES),
                   "seconds_per_rate": args.serve_seconds, "max_batch": max_batch, "budget_gb": SERVE_BUDGET / 2**30,
                   "latency": "arrival to pixels in the request's host buffer", "parallelism": "1 GPU"},
        "serving": points,
        "latency_at_rate": sla["rate"], "p50_ms": sla["batched"]["p50_ms"], "p95_ms": sla["batched"]["p95_ms"],
        "p99_ms": sla["batched"]["p99_ms"], "p99_1080p_ms": sla["batched"]["p99_1080p_ms"],
        "plain_p99_ms_at_rate": sla["plain"]["p99_ms"],
        "plain_max_frames_per_second": max(p["plain"]["frames_per_second"] for p in points),
        "e2e": {"value": top["frames_per_second"], "unit": "frames/s", "h2d_bytes_per_step": None,
                "d2h_bytes_per_step": None, "note": "every served frame ends in host memory"},
        "clocks": clk, "wall_s": wall,
    }
    for h in hs:
        R.free_scene(h)
    R.close()
    return line


def run_raycast(args, cfg) -> dict:
    """Ray queries (sft_raycast_instance, one GPU launch per step): 2^20 seeded rays against the
    instances of the atrium scene (the 262k-triangle atrium and four characters).  `value` with
    the rays resident in device memory (sftg_raycast_device), `e2e` through sftg_raycast with
    pinned host arrays (rays H2D, hits D2H inside the timed region)."""
    import torch
    import torch.distributed as dist
    from sofren2_gb300 import runtime, scenes

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    os.environ["SFT_CUDA_DEVICE"] = str(local)
    dev = torch.device("cuda", local)
    sc = getattr(scenes, cfg["gen"])()
    blob = sc.to_bytes()
    R = runtime.Renderer(640, 360, 1)
    h = R.load_scene(blob)
    n = cfg["rays"]
    rays = scenes.ray_batch(sc, n)
    ids = np.array([R.model_device_id(h, mi) for mi in range(len(sc.models))], np.int32)
    rays_dev = rays.copy()
    rays_dev["model"] = ids[rays["model"]]
    R.render_device(h, 0)                         # resident tables in place
    d_rays = torch.from_numpy(rays_dev.view(np.uint8).copy()).to(dev)
    d_hits = torch.empty(n * 32, dtype=torch.uint8, device=dev)
    pin_rays = torch.from_numpy(rays_dev.view(np.uint8).copy()).pin_memory()
    pin_hits = torch.empty(n * 32, dtype=torch.uint8).pin_memory()
    host_rays = pin_rays.numpy().view(runtime.RAY_DTYPE)
    host_hits = pin_hits.numpy().view(runtime.HIT_DTYPE)
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(R.stream(), device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def timed(step, k):
        times = []
        for _ in range(k):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        return times

    dev_step = lambda: R.raycast_device(d_rays.data_ptr(), n, d_hits.data_ptr())   # noqa: E731
    e2e_step = lambda: R.raycast_host(host_rays, host_hits)                         # noqa: E731
    for _ in range(args.warmup):
        dev_step()
        e2e_step()
    torch.cuda.synchronize()
    got = d_hits.cpu().numpy().view(runtime.HIT_DTYPE)
    assert got.tobytes() == host_hits.tobytes(), "device and host raycast entry points disagree"
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    dev_times = timed(dev_step, args.steps)
    e2e_times = timed(e2e_step, args.steps)
    clk = clocks.stop()
    ms_dev, ms_e2e = max_over_ranks([float(np.sum(dev_times)), float(np.sum(e2e_times))], device=f"cuda:{local}")
    peaks = _peaks()
    per_launch = float(np.mean(dev_times))
    alg = n * (96 + 32)
    achieved = alg / (per_launch * 1e-3) / 1e9
    line = {
        "metric": "rays_per_second", "value": job_throughput(args.steps * n, world, ms_dev), "unit": "rays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded rays against the seeded atrium scene)",
        "config": {"workload": cfg["name"], "rays": n, "hit_fraction": float((host_hits["hit"] == 1).mean()),
                   "l2": "flushed between steps (512 MiB device write, outside the timed events)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": job_throughput(args.steps * n, world, ms_e2e), "unit": "rays/s",
                "h2d_bytes_per_step": int(n * 96), "d2h_bytes_per_step": int(n * 32)},
        "gpu_launches": int(args.steps),
        "roofline": {"kernel": "k_raycast", "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": None, "algorithmic_bytes": alg,
                     "peak_source": peaks["src"],
                     "note": "latency-bound divergent BLAS walks; algorithmic bytes are the ray and hit records only"},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = raycast_cpu_baseline(blob, rays, seconds=args.cpu_seconds)
    R.free_scene(h)
    R.close()
    if world > 1:
        dist.destroy_process_group()
    return line if rank == 0 else None


def blas_scene(cfg):
    """The model whose BLAS is built (the atrium of the atrium scene: 7785 meshlets, 249120
    triangles), alone in a scene with one plain material, so creating it is meshlet upload and
    BLAS build only."""
    from sofren2_gb300 import scenes
    src = getattr(scenes, cfg["gen"])().models[cfg["model"]]
    sc = scenes.Scene()
    mat = sc.add_material(sc.add_texture(np.full((4, 4), 0xFFFFFFFF, np.uint32)))
    sc.add_model(scenes.Model(src.meshes, [mat] * len(src.meshes)))
    sc.frames.append(scenes._camera_frame(64, 64))
    return sc


def run_blas(args, cfg) -> dict:
    """BLAS construction (sft__blas_build_model) on the device, one build per step.  `value`:
    triangles/s over the build's span on the upload stream between two CUDA events (meshlets
    already resident: the build starts after their upload has finished).  `e2e`: sft_model_create
    from host meshlet arrays (scene load: meshlet upload + build + root read-back), wall clock
    around the synchronous call, which returns with the model resident."""
    import torch
    import torch.distributed as dist
    from sofren2_gb300 import runtime

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    os.environ["SFT_CUDA_DEVICE"] = str(local)
    sc = blas_scene(cfg)
    blob = sc.to_bytes()
    ms = sc.models[0].meshes
    n_meshlets = sum(m.n for m in ms)
    R = runtime.Renderer(64, 64, 1)
    for _ in range(args.warmup):
        R.free_scene(R.load_scene(blob))
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    stream_ms, wall_ms, build_wall = [], [], []
    st = {}
    for _ in range(args.steps):
        t0 = time.perf_counter()
        h = R.load_scene(blob)
        wall_ms.append(1e3 * (time.perf_counter() - t0))
        st = R.last_blas_build()
        stream_ms.append(st["stream_ms"])
        build_wall.append(st["wall_ms"])
        R.free_scene(h)
    clk = clocks.stop()
    ms_dev, ms_e2e = max_over_ranks([float(np.sum(stream_ms)), float(np.sum(wall_ms))], device=f"cuda:{local}")
    tris = st["triangles"]
    h = R.load_scene(blob)
    n_nodes = len(R.model_blas(h, 0)[0]) // 256
    R.free_scene(h)
    peaks = _peaks()
    alg = n_meshlets * (2560 + 512) + n_nodes * 256
    per_build = float(np.mean(stream_ms))
    achieved = alg / (per_build * 1e-3) / 1e9
    line = {
        "metric": "triangles_per_second", "value": job_throughput(args.steps * tris, world, ms_dev), "unit": "triangles/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (the seeded atrium model)",
        "config": {"workload": cfg["name"], "meshlets": n_meshlets, "triangles": tris, "nodes": n_nodes,
                   "l2": "inputs of 24 MB written by the upload just before each build (L2-resident, as at model creation)",
                   "parallelism": f"replicas x{world}", "host_wall_ms_per_build": float(np.mean(build_wall))},
        "e2e": {"value": job_throughput(args.steps * tris, world, ms_e2e), "unit": "triangles/s",
                "h2d_bytes_per_step": int(n_meshlets * (2560 + 512 + 32)), "d2h_bytes_per_step": 256},
        "gpu_launches": int(st["launches"]) * args.steps,
        "roofline": {"kernel": "BLAS build (all kernels)", "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": None, "algorithmic_bytes": alg,
                     "peak_source": peaks["src"],
                     "note": "latency bound: 15 dependent sort levels and host reads of the work-list counters; "
                             "algorithmic bytes are the meshlet positions and indices read and the node images written"},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = blas_cpu_baseline(blob, tris, seconds=args.cpu_seconds)
    R.close()
    if world > 1:
        dist.destroy_process_group()
    return line if rank == 0 else None


def run_pose(args, cfg) -> dict:
    """Skeletal poses (sft_pose_update, one warp per request): 2^16 seeded (animation, time)
    requests on the 22-bone rig, posed and global matrices out.  `value` through
    sftg_pose_eval_device with requests and outputs in device memory; `e2e` through sftg_pose_eval
    with page-locked host arrays (requests H2D, matrices D2H inside the timed region)."""
    import torch
    import torch.distributed as dist
    from sofren2_gb300 import runtime, scenes

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    os.environ["SFT_CUDA_DEVICE"] = str(local)
    dev = torch.device("cuda", local)
    rig = scenes.pose_rig()
    nb = len(rig["bones"])
    n = cfg["requests"]
    req = scenes.pose_requests(rig, n, seed=8)
    R = runtime.Renderer(64, 64, 1)
    sk = R.skeleton_upload(rig)
    rec = np.zeros(n, runtime.POSE_REQUEST_DTYPE)
    rec["skeleton"] = sk
    rec["animation"] = [a for a, _ in req]
    rec["time"] = [t for _, t in req]
    off = (np.arange(n, dtype=np.uint32) * nb).astype(np.uint32)
    d_req = torch.from_numpy(rec.view(np.uint8).copy()).to(dev)
    d_off = torch.from_numpy(off.view(np.uint8).copy()).to(dev)
    d_posed = torch.zeros(n * nb * 16, dtype=torch.float32, device=dev)
    d_glob = torch.zeros(n * nb * 16, dtype=torch.float32, device=dev)
    pin_req = torch.from_numpy(rec.view(np.uint8).copy()).pin_memory()
    pin_posed = torch.zeros(n * nb * 16, dtype=torch.float32).pin_memory()
    pin_glob = torch.zeros(n * nb * 16, dtype=torch.float32).pin_memory()
    host_req = pin_req.numpy().view(runtime.POSE_REQUEST_DTYPE)
    host_posed, host_glob = pin_posed.numpy(), pin_glob.numpy()
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(R.stream(), device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def timed(step, k):
        times = []
        for _ in range(k):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        return times

    dev_step = lambda: R.pose_eval_device(d_req.data_ptr(), d_off.data_ptr(), n, d_posed.data_ptr(), d_glob.data_ptr())   # noqa: E731
    e2e_step = lambda: R.pose_eval_host(host_req, host_posed, host_glob)                                                  # noqa: E731
    for _ in range(args.warmup):
        dev_step()
        e2e_step()
    torch.cuda.synchronize()
    assert d_posed.cpu().numpy().tobytes() == host_posed.tobytes(), "device and host pose entry points disagree"
    assert d_glob.cpu().numpy().tobytes() == host_glob.tobytes(), "device and host pose entry points disagree"
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    dev_times = timed(dev_step, args.steps)
    e2e_times = timed(e2e_step, args.steps)
    clk = clocks.stop()
    ms_dev, ms_e2e = max_over_ranks([float(np.sum(dev_times)), float(np.sum(e2e_times))], device=f"cuda:{local}")
    peaks = _peaks()
    per_launch = float(np.mean(dev_times))
    alg = n * (12 + 4 + 2 * nb * 64)
    achieved = alg / (per_launch * 1e-3) / 1e9
    valid = int(((rec["animation"] >= 0) & (rec["animation"] < len(rig["anims"]))).sum())
    line = {
        "metric": "poses_per_second", "value": job_throughput(args.steps * n, world, ms_dev), "unit": "poses/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded rig and requests)",
        "config": {"workload": cfg["name"], "requests": n, "bones": nb, "animations": len(rig["anims"]),
                   "requests_in_range": valid,
                   "l2": "flushed between steps (512 MiB device write, outside the timed events); outputs 184 MB per step",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": job_throughput(args.steps * n, world, ms_e2e), "unit": "poses/s",
                "h2d_bytes_per_step": int(n * 12), "d2h_bytes_per_step": int(2 * n * nb * 64)},
        "gpu_launches": int(args.steps),
        "roofline": {"kernel": "k_pose", "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": None, "algorithmic_bytes": alg,
                     "peak_source": peaks["src"],
                     "note": "algorithmic bytes: request, offset and the posed and global matrices written; keys read from L2"},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = pose_cpu_baseline(rig, req, seconds=args.cpu_seconds)
    R.close()
    if world > 1:
        dist.destroy_process_group()
    return line if rank == 0 else None


def pose_cpu_baseline(rig: dict, req: list, seconds: float = 12.0, chunk: int = 4096) -> dict:
    """The oracle's restated sft_pose_update (bit-identical to the reference's) on one host core,
    over consecutive chunks of the same requests until `seconds` have passed."""
    from oracle_lib import build_oracle, oracle_pose, pose_blob
    build_oracle()
    nb = len(rig["bones"])
    done, t = 0, 0.0
    while t < seconds and done < len(req):
        part = req[done:done + chunk]
        blob = pose_blob(rig, part)
        t0 = time.perf_counter()
        oracle_pose(blob, nb, len(part))
        t += time.perf_counter() - t0
        done += len(part)
    return {"value": done / t, "unit": "poses/s", "cores": 1, "kind": "port",
            "sample": f"the first {done} requests of the same set (oracle/sft_oracle.c sfto_pose_eval, one thread, as "
                      "the reference's sft_pose_update runs on the calling thread)"}


def blas_cpu_baseline(blob: bytes, tris: int, seconds: float = 12.0) -> dict:
    """The oracle's restated BLAS builder (the reference's recursive build, one thread) on the
    same model, repeated until `seconds` have passed."""
    from oracle_lib import Oracle, build_oracle
    build_oracle()
    o = Oracle(blob)
    times = []
    try:
        t_end = time.perf_counter() + seconds
        while time.perf_counter() < t_end or len(times) < 2:
            t0 = time.perf_counter()
            o.blas_rebuild(0, 1)
            times.append(time.perf_counter() - t0)
            if len(times) >= 500:
                break
    finally:
        o.close()
    return {"value": tris * len(times) / sum(times), "unit": "triangles/s", "cores": 1, "kind": "port",
            "sample": f"{len(times)} builds of the same model (oracle/sft_oracle.c blas_build, one thread, as the "
                      "reference builds at load time on the calling thread)"}


def raycast_cpu_baseline(blob: bytes, rays: np.ndarray, seconds: float = 12.0, chunk: int = 1 << 15) -> dict:
    """The oracle's scalar sft_raycast_instance restatement on one host core, over consecutive
    chunks of the same rays until `seconds` have passed."""
    from oracle_lib import Oracle, build_oracle
    build_oracle()
    o = Oracle(blob)
    done, t = 0, 0.0
    try:
        while t < seconds and done < len(rays):
            r = rays[done:done + chunk]
            t0 = time.perf_counter()
            o.raycast(r)
            t += time.perf_counter() - t0
            done += len(r)
    finally:
        o.close()
    return {"value": done / t, "unit": "rays/s", "cores": 1, "kind": "port",
            "sample": f"the first {done} rays of the same batch (oracle/sft_oracle.c sfto_raycast, one thread, as "
                      "the reference's sft_raycast_instance runs on the calling thread)"}


def reference_frame_times(blob: bytes, samples: int, frame: int = 0, threads: int | None = None, repeat: int = 100000,
                          seconds: float = 0.0) -> np.ndarray | None:
    """Wall times (s) of whole frames (lights, camera, draws, sft_present) of the reference's own
    render path: sofren2.c unmodified, built for this host by `make -C oracle ref_bench` (the NEON
    path on aarch64, AVX2 on x86-64), run with its own worker pool, sft_init(w, h, threads).
    `repeat` frames, or fewer once `seconds` have passed (at least 3).  None when that build is
    absent on this host."""
    import tempfile
    exe = os.path.join(ROOT, "oracle", "_ref", f"ref_bench_{samples}x")
    if not os.path.exists(exe):
        return None
    threads = threads or os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as td:
        sp, tp = os.path.join(td, "scene.sfts"), os.path.join(td, "times.bin")
        with open(sp, "wb") as f:
            f.write(blob)
        env = dict(os.environ, SFT_NO_DUMP="1", SFT_TIMES=tp)
        if seconds > 0:
            env["SFT_TIME_BUDGET_MS"] = str(int(seconds * 1e3))
        r = subprocess.run([exe, sp, os.devnull, str(frame), str(threads), str(repeat)], env=env, capture_output=True, text=True)
        if r.returncode != 0 or not os.path.exists(tp):
            return None
        return np.fromfile(tp, np.uint64).astype(np.float64) * 1e-9


_REF_AGREEMENT: dict = {}


def reference_agreement(blob: bytes, samples: int, width: int, height: int, frame: int = 0) -> float:
    """Fraction of the pixels of the reference build's frame (ref_bench, one dumped render) within
    4 LSB per channel of the oracle's frame, which equals the GPU's bit for bit (0 when the mean
    difference exceeds REF_MEAN_LSB_MAX).  A build that renders something else (a broken SIMD
    path) must not be timed as the baseline."""
    import hashlib
    import tempfile
    from oracle_io import read_dump
    from oracle_lib import Oracle, build_oracle
    key = (hashlib.sha1(blob).hexdigest(), samples, frame)
    if key not in _REF_AGREEMENT:
        exe = os.path.join(ROOT, "oracle", "_ref", f"ref_bench_{samples}x")
        close = 0.0
        with tempfile.TemporaryDirectory() as td:
            sp, dp = os.path.join(td, "scene.sfts"), os.path.join(td, "r.dump")
            with open(sp, "wb") as f:
                f.write(blob)
            r = subprocess.run([exe, sp, dp, str(frame), str(os.cpu_count() or 1)], capture_output=True)
            if r.returncode == 0:
                ref = read_dump(dp)[0]["color"].reshape(-1)
                build_oracle()
                o = Oracle(blob)
                try:
                    ours, _, _ = o.render_color(frame, samples, width, height, threads=os.cpu_count() or 1)
                finally:
                    o.close()
                ours = np.asarray(ours).reshape(-1)
                if ours.size == ref.size:
                    a = np.stack([(ref >> k) & 0xFF for k in (16, 8, 0)]).astype(np.int32)
                    b = np.stack([(ours >> k) & 0xFF for k in (16, 8, 0)]).astype(np.int32)
                    close = float((np.abs(a - b).max(axis=0) <= 4).mean())
                    if np.abs(a - b).mean() > REF_MEAN_LSB_MAX:
                        close = 0.0
        _REF_AGREEMENT[key] = close
    return _REF_AGREEMENT[key]


# The reference build renders the same frame: most pixels within 4 LSB per channel of the oracle's
# and a small mean difference.  Its own platform differences stay below these: its NEON path
# traces 4-wide proxy batches (other packet frustums, so some light visibility and shadows differ)
# and groups pixels 2x2 for LOD and the shadow block rule (atrium 1080p 4x: 86.7 % within 4 LSB,
# mean 3.2 LSB; skinned 1080p 2x: 99.0 %, 0.10).  A broken build (an empty frame) falls far below.
REF_AGREEMENT_MIN = 0.80
REF_MEAN_LSB_MAX = 8.0


def _reference_desc(threads: int) -> str:
    import platform
    if platform.machine() == "aarch64":
        build = ("its NEON path, 4 lanes, gcc -O2 -flax-vector-conversions, two defects repaired at build time: "
                 "the call GCC 13 rejects (vmovl_u16 of a uint16x8_t, sofren2.c:473) gets its low half, and "
                 "sft_vf_fmsub's sign (c - a*b instead of a*b - c, sofren2.c:425) is corrected")
    else:
        build = "its AVX2 path, 8 lanes, gcc -O2 -mavx2 -mfma"
    return (f"the reference's own code (sofren2.c, source unmodified; {build}) on {platform.machine()} with "
            f"sft_init(w, h, {threads}), wall time of whole frames")


def reference_frames(blob: bytes, samples: int, width: int, height: int, seconds: float, frame: int = 0,
                     threads: int | None = None) -> dict | None:
    """The reference's own render path timed on the host cores: frames/s over frames 2..N.  None
    when its build is absent here or renders a frame that disagrees with the oracle's."""
    threads = threads or os.cpu_count() or 1
    if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", f"ref_bench_{samples}x")):
        return None
    agree = reference_agreement(blob, samples, width, height, frame)
    if agree < REF_AGREEMENT_MIN:
        return None
    t = reference_frame_times(blob, samples, frame, threads, seconds=seconds)
    if t is None:
        return None
    steady = t[1:] if t.size > 1 else t
    return {"value": float(steady.size / steady.sum()), "unit": "frames/s", "cores": threads, "kind": "reference",
            "agreement": f"{agree:.5f} of its pixels within 4 LSB of the oracle's (= the GPU's) frame",
            "sample": f"{steady.size} frames of the same workload after 1 untimed frame: {_reference_desc(threads)}"}


def cpu_baseline(blob: bytes, samples: int, width: int, height: int, seconds: float = 12.0, frame: int = 0) -> dict:
    """The reference's own CPU path timed on the host cores when it is built on this host, with the
    oracle port's number beside it; the oracle port alone otherwise."""
    ref = reference_frames(blob, samples, width, height, seconds * 0.6, frame)
    port = port_frames(blob, samples, width, height, seconds * (0.4 if ref else 1.0), frame)
    if ref is None:
        return port
    ref["port"] = {k: port[k] for k in ("value", "unit", "cores", "kind", "sample")}
    return ref


def port_frames(blob: bytes, samples: int, width: int, height: int, seconds: float = 12.0, frame: int = 0) -> dict:
    """The oracle restatement of the reference algorithm, timed on the host cores."""
    from oracle_lib import Oracle, build_oracle
    build_oracle()
    threads = os.cpu_count() or 1
    o = Oracle(blob)
    try:
        times = []
        t_end = time.perf_counter() + seconds
        while time.perf_counter() < t_end or len(times) < 2:
            t0 = time.perf_counter()
            o.render_color(frame, samples, width, height, threads=threads)
            times.append(time.perf_counter() - t0)
            if len(times) >= 200:
                break
    finally:
        o.close()
    steady = times[1:] if len(times) > 1 else times
    fps = len(steady) / sum(steady)
    return {"value": fps, "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"{len(steady)} frames of the same workload after 1 untimed frame "
                      f"(oracle/sft_oracle.c, tile-parallel over {threads} threads)"}


def run_reference(args, cfg) -> dict | None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    from sofren2_gb300 import scenes
    from oracle_lib import Oracle, build_oracle
    build_oracle()
    threads = os.cpu_count() or 1
    if args.config == 6:   # bounded sample: 2^15 rays per step, consecutive chunks of the batch
        sc = getattr(scenes, cfg["gen"])()
        rays = scenes.ray_batch(sc, cfg["rays"])
        o = Oracle(sc.to_bytes())
        chunk, times = 1 << 15, []
        try:
            for k in range(max(1, args.warmup) + args.steps):
                r = rays[(k * chunk) % len(rays):][:chunk]
                t0 = time.perf_counter()
                o.raycast(r)
                if k >= max(1, args.warmup):
                    times.append((time.perf_counter() - t0) / len(r))
        finally:
            o.close()
        rps = len(times) / sum(times)
        return {"metric": "rays_per_second", "value": rps, "unit": "rays/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * chunk / rps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded rays against the seeded atrium scene)", "impl": "reference",
                "config": {"workload": cfg["name"], "rays": cfg["rays"], "sample": f"{chunk} rays per step"},
                "cpu_baseline": {"value": rps, "unit": "rays/s", "cores": 1, "kind": "port",
                                 "sample": f"{len(times)} steps of {chunk} rays after {max(1, args.warmup)} warm-up, scalar "
                                           "restatement of sft_raycast_instance (oracle/sft_oracle.c), one thread"},
                "e2e": {"value": rps, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.config == 8:   # bounded sample: 4096 requests per step, consecutive chunks of the set
        from oracle_lib import oracle_pose, pose_blob
        rig = scenes.pose_rig()
        nb = len(rig["bones"])
        req = scenes.pose_requests(rig, cfg["requests"], seed=8)
        chunk, times = 4096, []
        for k in range(max(1, args.warmup) + args.steps):
            part = req[(k * chunk) % len(req):][:chunk]
            blob = pose_blob(rig, part)
            t0 = time.perf_counter()
            oracle_pose(blob, nb, len(part))
            if k >= max(1, args.warmup):
                times.append((time.perf_counter() - t0) / len(part))
        pps = len(times) / sum(times)
        return {"metric": "poses_per_second", "value": pps, "unit": "poses/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * chunk / pps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded rig and requests)", "impl": "reference",
                "config": {"workload": cfg["name"], "requests": cfg["requests"], "sample": f"{chunk} requests per step"},
                "cpu_baseline": {"value": pps, "unit": "poses/s", "cores": 1, "kind": "port",
                                 "sample": f"{len(times)} steps of {chunk} requests after {max(1, args.warmup)} warm-up, "
                                           "restated sft_pose_update (oracle/sft_oracle.c), one thread"},
                "e2e": {"value": pps, "unit": "poses/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.config == 7:   # each step one build of the same model
        sc = blas_scene(cfg)
        o = Oracle(sc.to_bytes())
        tris = sum(int(m.tri_count.sum()) for m in sc.models[0].meshes)
        times = []
        try:
            for k in range(max(1, args.warmup) + args.steps):
                t0 = time.perf_counter()
                o.blas_rebuild(0, 1)
                if k >= max(1, args.warmup):
                    times.append(time.perf_counter() - t0)
        finally:
            o.close()
        tps = tris * len(times) / sum(times)
        return {"metric": "triangles_per_second", "value": tps, "unit": "triangles/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (the seeded atrium model)", "impl": "reference",
                "config": {"workload": cfg["name"], "triangles": tris},
                "cpu_baseline": {"value": tps, "unit": "triangles/s", "cores": 1, "kind": "port",
                                 "sample": f"{len(times)} builds after {max(1, args.warmup)} warm-up, restated recursive builder "
                                           "(oracle/sft_oracle.c), one thread"},
                "e2e": {"value": tps, "unit": "triangles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.config == 5:   # bounded sample: the first frame of each scene, cycling
        scs, smp = scenes.config5()
        jobs = [(sc.to_bytes(), 0, S, sc.frames[0].width, sc.frames[0].height) for sc, S in zip(scs, smp)]
    elif args.config == 4:   # bounded sample: one view per step, cycling over the scenes
        scs, vlist = scenes.config4()
        picks = [next(v for v in vlist if v[0] == si) for si in range(len(scs))]
        jobs = [(scs[si].to_bytes(), f, S, scs[si].frames[f].width, scs[si].frames[f].height) for si, f, S in picks]
    else:
        jobs = [(getattr(scenes, cfg["gen"])().to_bytes(), 0, cfg["samples"], cfg["width"], cfg["height"])]
    # the reference's own build when this host has it (each job: its warm-up frames, then its
    # share of the K timed frames, in one process with the reference's worker pool)
    times, kind = [], "reference"
    warm = max(1, args.warmup)
    agree = []
    for j, (blob, f, S, w, h) in enumerate(jobs):
        n = len(range(j, args.steps, len(jobs)))
        if n == 0:
            continue
        t = None
        if os.path.exists(os.path.join(ROOT, "oracle", "_ref", f"ref_bench_{S}x")):
            agree.append(reference_agreement(blob, S, w, h, f))
            if agree[-1] >= REF_AGREEMENT_MIN:
                t = reference_frame_times(blob, S, f, threads, repeat=warm + n)
        if t is None or t.size < warm + n:
            times, kind = [], "port"
            break
        times.extend(t[warm:].tolist())
    if kind == "port":
        oracles = [Oracle(j[0]) for j in jobs]
        try:
            for k in range(warm):
                _, f, S, w, h = jobs[k % len(jobs)]
                oracles[k % len(jobs)].render_color(f, S, w, h, threads=threads)
            for k in range(args.steps):
                _, f, S, w, h = jobs[k % len(jobs)]
                t0 = time.perf_counter()
                oracles[k % len(jobs)].render_color(f, S, w, h, threads=threads)
                times.append(time.perf_counter() - t0)
        finally:
            for o in oracles:
                o.close()
        why = ("absent on this host" if not agree else
               f"renders frames that disagree with the oracle's ({min(agree):.4f} of pixels within 4 LSB, or a large mean difference)")
        sample = (f"{len(times)} frames after {warm} warm-up, CPU restatement of the reference algorithm "
                  f"(oracle/sft_oracle.c), tile-parallel; the reference's own build is {why}")
    else:
        sample = f"{len(times)} frames after {warm} warm-up frames per scene: {_reference_desc(threads)}"
    fps = len(times) / sum(times)
    return {"metric": "frames_per_second", "value": fps, "unit": "frames/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scene)", "impl": "reference",
            "config": frame_config(cfg) if args.config < 4 else {"workload": cfg["name"], "sample": "one view per step, cycling over the scenes"},
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def frame_config(cfg) -> dict:
    """The config dict of a single-view frame workload, the same in both arms."""
    return {"workload": cfg["name"], "width": cfg["width"], "height": cfg["height"], "msaa": cfg["samples"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=2, choices=sorted(CONFIGS))
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--serve-seconds", type=float, default=3.0, help="config 5: seconds of arrivals per rate")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    cfg = CONFIGS[args.config]
    if args.impl == "reference":
        line = run_reference(args, cfg)
    elif args.config == 4:
        line = run_batch(args, cfg)
    elif args.config == 5:
        line = run_serve(args, cfg)
    elif args.config == 6:
        line = run_raycast(args, cfg)
    elif args.config == 7:
        line = run_blas(args, cfg)
    elif args.config == 8:
        line = run_pose(args, cfg)
    else:
        line = run_ours(args, cfg)
    if line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
