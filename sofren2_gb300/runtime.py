"""ctypes front end of libsofren2_gb300.so: the sft_* API plus the scene player.

The library is the only rendering path.  Loading fails loudly when it has not been built
or when no CUDA device is present; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_LIB = None


class SftgDebugOut(C.Structure):
    """struct sftg_debug_out (include/sftg.h)."""
    _fields_ = [
        ("vis_depth", C.c_void_p), ("vis_id", C.c_void_p), ("tile_counts", C.c_void_p),
        ("tile_payloads", C.c_void_p), ("tile_payload_cap", C.c_uint64), ("tile_payload_total", C.c_void_p),
        ("ss_cache", C.c_void_p), ("light_vis", C.c_void_p), ("clip_tris", C.c_void_p), ("clip_cap", C.c_uint64),
        ("clip_total", C.c_void_p), ("shadow", C.c_void_p), ("status", C.c_void_p),
    ]


def library_path() -> str:
    return _build.LIB


def load_library(build_if_missing: bool = True) -> C.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run `python -m sofren2_gb300.build` first")
        _build.build_library()
    lib = C.CDLL(path)
    v, i32, u32, u64, f32, p = None, C.c_int32, C.c_uint32, C.c_uint64, C.c_float, C.c_void_p
    sig = {
        "sft_init": (v, [i32, i32, i32]), "sft_release": (v, []), "sft_set_msaa_samples": (v, [i32]),
        "sft_get_last_error": (C.c_char_p, []), "sft_set_debug_capture": (v, [p]),
        "sft_get_frame_timings": (v, [p]), "sftx_scene_load": (p, [p, u64]), "sftx_scene_free": (v, [p]),
        "sftx_scene_frame_count": (u32, [p]), "sftx_scene_render": (i32, [p, u32, p, i32]),
        "sftx_scene_frame_size": (u32, [p, u32, p, p]), "sft_get_launch_count": (i32, []),
        "sft_get_cuda_stream": (p, []), "sft_set_debug_mode": (v, [i32]),
        "sftx_scene_render_batch": (i32, [p, p, p, u32, p, p]),
        "sftx_scene_autotune_batch": (i32, [p, p, p, u32, i32]),
        "sftx_scene_render_ex": (i32, [p, u32, p, i32, u32]),
        "sftx_serve": (i32, [p, p, u32, u32, u64, i32, p, u32, p, p, p]),
        "sftx_serve_ex": (i32, [p, p, u32, u32, u64, i32, u32, p, u32, p, p, p]),
        "sftx_serve_warm": (i32, [p, p, u32, u32, u64, u32, p, u32]),
        "sft_get_gpu_context": (p, []), "sftg_get_tuning": (i32, [p, p]), "sftg_set_tuning": (i32, [p, p]),
        "sftg_skeleton_upload": (i32, [p, p, u32, p, u32, p]), "sftg_pose_eval": (i32, [p, p, u32, p, p]),
        "sftg_last_error": (C.c_char_p, [p]), "sftx_scene_model": (p, [p, u32]),
        "sft_raycast_batch": (v, [p, p, p, p, u32, p]), "sftg_raycast": (i32, [p, p, u32, p]),
        "sftg_raycast_device": (i32, [p, p, u32, p]),
        "sft_batch_begin": (v, []), "sft_batch_submit": (i32, []), "sft_batch_submit_async": (i32, [u32]),
        "sft_batch_done": (i32, [u32]), "sft_batch_wait": (i32, [u32]),
        "sftx_scene_render_lanes": (i32, [p, p, p, u32, p, p, u32]), "sftg_launch_total": (u64, [p]),
        "sft_model_get_blas": (p, [p, p, p]), "sftg_pose_eval_device": (i32, [p, p, p, u32, p, p]), "sftg_last_blas_build": (i32, [p, p, p, p, p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    _LIB = lib
    return lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class SftgBoneDesc(C.Structure):
    _fields_ = [("inverse_bind", C.c_float * 16), ("local_bind", C.c_float * 16), ("parent", C.c_int32),
                ("base_t", C.c_float * 3), ("base_r", C.c_float * 4), ("base_s", C.c_float * 3)]


class SftgSamplerDesc(C.Structure):
    _fields_ = [("inputs", C.c_void_p), ("outputs", C.c_void_p), ("count", C.c_int32), ("is_step", C.c_int32)]


class SftgChannelDesc(C.Structure):
    _fields_ = [("sampler", C.c_int32), ("node", C.c_int32), ("path", C.c_int32)]


class SftgAnimationDesc(C.Structure):
    _fields_ = [("samplers", C.c_void_p), ("channels", C.c_void_p), ("sampler_count", C.c_int32),
                ("channel_count", C.c_int32), ("duration", C.c_float)]


class SftgPoseRequest(C.Structure):
    _fields_ = [("skeleton", C.c_int32), ("animation", C.c_int32), ("time", C.c_float)]


POSE_REQUEST_DTYPE = np.dtype([("skeleton", "<i4"), ("animation", "<i4"), ("time", "<f4")])


# sftg_ray / sftg_ray_hit records (include/sftg.h)
RAY_DTYPE = np.dtype([("T", "<f4", (16,)), ("o", "<f4", (3,)), ("d", "<f4", (3,)), ("max_dist", "<f4"), ("model", "<i4")])
HIT_DTYPE = np.dtype([("hit", "<u4"), ("dist", "<f4"), ("pos", "<f4", (3,)), ("nrm", "<f4", (3,))])


class SftInstance(C.Structure):
    """sft_instance (include/sofren2.h, sofren2.c:1198-1203)."""
    _fields_ = [("model", C.c_void_p), ("transform", C.c_float * 16), ("ss_meshlet_offset", C.c_uint32),
                ("posed_bone_matrices", C.c_void_p)]


class SftRayHit(C.Structure):
    """sft_ray_hit (sofren2.c:895-900)."""
    _fields_ = [("hit", C.c_uint8), ("distance", C.c_float), ("pos", C.c_float * 3), ("normal", C.c_float * 3)]


class SftxRequest(C.Structure):
    """struct sftx_request (sofren2_gb300/csrc/sft_serve.c)."""
    _fields_ = [("arrival_ns", C.c_uint64), ("device_bytes", C.c_uint64), ("scene", C.c_uint32), ("frame", C.c_uint32),
                ("samples", C.c_int32), ("max_point_lights", C.c_uint32)]


class SftxServeStats(C.Structure):
    _fields_ = [("batches", C.c_uint64), ("max_batch", C.c_uint64), ("peak_bytes", C.c_uint64), ("errors", C.c_uint64),
                ("max_inflight", C.c_uint64)]


# struct sftg_tuning (include/sftg.h), field by field in order: (name, int32 count)
TUNING_LAYOUT = (("resolve_split", 3), ("raster_slab_rows", 3), ("geom_job_width", 1), ("occl_ray_prune", 1),
                 ("raster_bands", 3), ("tile_lights", 3), ("tile_queue", 1))


def request_device_bytes(width: int, height: int, samples: int, meshlets: int) -> int:
    """Device memory a request holds while in flight: visibility buffer (8 B per sample), colour,
    screen-space cache and batch records per meshlet, tile lists and clip pool at a generous
    estimate."""
    tiles = ((width + 63) // 64) * ((height + 63) // 64)
    return tiles * samples * 4096 * 8 + width * height * 4 + meshlets * (3328 + 16 * 16 + 16 * 8 + 16) + tiles * 64 * 1024


class Renderer:
    """One GPU renderer (the reference's sft_state singleton)."""

    _live = False

    def __init__(self, width: int, height: int, samples: int = 1):
        if Renderer._live:
            raise RuntimeError("only one Renderer may exist at a time (the sft_* API keeps global state)")
        self.lib = load_library()
        self.lib.sft_init(width, height, 0)
        self.lib.sft_set_msaa_samples(samples)
        self.samples = samples
        Renderer._live = True

    def close(self):
        if Renderer._live:
            self.lib.sft_release()
            Renderer._live = False

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_debug_mode(self, mode: int):
        """enum sft_debug_mode: 0 none, 1 wireframe, 2 tiles, 3 depth, 4 light count, 5 checkerboard."""
        self.lib.sft_set_debug_mode(mode)

    def set_samples(self, samples: int):
        self.lib.sft_set_msaa_samples(samples)
        self.samples = samples

    def load_scene(self, blob: bytes):
        buf = np.frombuffer(blob, dtype=np.uint8)
        h = self.lib.sftx_scene_load(_ptr(buf), len(blob))
        if not h:
            raise RuntimeError("scene blob rejected: " + (self.lib.sft_get_last_error() or b"").decode())
        return h

    def free_scene(self, h):
        self.lib.sftx_scene_free(h)

    def frame_size(self, h, frame: int) -> tuple[int, int]:
        w, hh = C.c_uint32(), C.c_uint32()
        self.lib.sftx_scene_frame_size(h, frame, C.byref(w), C.byref(hh))
        return w.value, hh.value

    def render_device(self, h, frame: int = 0) -> None:
        """Renders with the colour left in device memory (no pixel copy to the host)."""
        rc = self.lib.sftx_scene_render(h, frame, None, 0)
        if rc != 0:
            raise RuntimeError("render failed: " + (self.lib.sft_get_last_error() or b"").decode())

    def stream(self) -> int:
        return self.lib.sft_get_cuda_stream() or 0

    def launch_total(self) -> int:
        """Kernels launched by every batch finished so far, on all submission lanes."""
        return int(self.lib.sftg_launch_total(self.lib.sft_get_gpu_context()))

    def launch_count(self) -> int:
        return int(self.lib.sft_get_launch_count())

    def timings(self) -> np.ndarray:
        t = np.zeros(5, np.float32)
        self.lib.sft_get_frame_timings(_ptr(t))
        return t

    def render(self, h, frame: int = 0, color: np.ndarray | None = None) -> np.ndarray:
        w, hh = self.frame_size(h, frame)
        if color is None:
            color = np.zeros((hh, w), dtype=np.uint32)
        rc = self.lib.sftx_scene_render(h, frame, _ptr(color), color.strides[0])
        err = self.lib.sft_get_last_error()
        if rc != 0:
            raise RuntimeError("render failed: " + (err or b"").decode())
        return color

    def render_batch(self, views: list[tuple], colors: list[np.ndarray | None] | None = None,
                     lanes: int = 0) -> list[np.ndarray | None]:
        """Renders views [(scene handle, frame, samples), ...] in one batched submission, or with
        lanes >= 1 as that many batches overlapping on submission lanes 1..lanes.

        colors: None (every colour stays on the device) or one array (or None) per view; a
        missing array is allocated.  Returns the per-view colour arrays (None for device-only)."""
        n = len(views)
        hs = (C.c_void_p * n)(*[h for h, _, _ in views])
        fr = np.array([f for _, f, _ in views], np.uint32)
        sm = np.array([s for _, _, s in views], np.int32)
        out: list[np.ndarray | None] = [None] * n
        cp = None
        pitch = None
        if colors is not None:
            ptrs = (C.c_void_p * n)()
            pitch = np.zeros(n, np.int32)
            for i, (h, f, _) in enumerate(views):
                c = colors[i]
                if c is None:
                    w, hh = self.frame_size(h, f)
                    c = np.zeros((hh, w), np.uint32)
                out[i] = c
                ptrs[i] = c.ctypes.data
                pitch[i] = c.strides[0]
            cp = ptrs
        if lanes:
            rc = self.lib.sftx_scene_render_lanes(hs, _ptr(fr), _ptr(sm), n, cp, _ptr(pitch), lanes)
        else:
            rc = self.lib.sftx_scene_render_batch(hs, _ptr(fr), _ptr(sm), n, cp, _ptr(pitch))
        self.lib.sft_set_msaa_samples(self.samples)
        if rc != 0:
            raise RuntimeError("batch render failed: " + (self.lib.sft_get_last_error() or b"").decode())
        return out

    def autotune_batch(self, views: list[tuple], reps: int = 5) -> dict:
        """Tunes the scheduling knobs (sftg_autotune) on views [(scene handle, frame, samples)]
        rendered as one batch; returns the chosen setting."""
        n = len(views)
        hs = (C.c_void_p * n)(*[h for h, _, _ in views])
        fr = np.array([f for _, f, _ in views], np.uint32)
        sm = np.array([s for _, _, s in views], np.int32)
        rc = self.lib.sftx_scene_autotune_batch(hs, _ptr(fr), _ptr(sm), n, reps)
        self.lib.sft_set_msaa_samples(self.samples)
        if rc != 0:
            raise RuntimeError("autotune failed: " + (self.lib.sft_get_last_error() or b"").decode())
        return self.tuning()

    def tuning(self) -> dict:
        t = np.zeros(sum(n for _, n in TUNING_LAYOUT), np.int32)
        self.lib.sftg_get_tuning(self.lib.sft_get_gpu_context(), _ptr(t))
        out, k = {}, 0
        for name, n in TUNING_LAYOUT:
            out[name] = t[k:k + n].tolist() if n > 1 else int(t[k])
            k += n
        return out

    def set_tuning(self, resolve_split=(16, 8, 16), raster_slab_rows=(8, 8, 4), geom_job_width=1, occl_ray_prune=0,
                   raster_bands=(0, 0, 0), tile_lights=(0, 0, 0), tile_queue=0) -> None:
        vals = dict(resolve_split=resolve_split, raster_slab_rows=raster_slab_rows, geom_job_width=geom_job_width,
                    occl_ray_prune=occl_ray_prune, raster_bands=raster_bands, tile_lights=tile_lights, tile_queue=tile_queue)
        flat = []
        for name, n in TUNING_LAYOUT:
            v = vals[name]
            flat += list(v) if n > 1 else [v]
        t = np.array(flat, np.int32)
        if self.lib.sftg_set_tuning(self.lib.sft_get_gpu_context(), _ptr(t)) != 0:
            raise ValueError("tuning out of range")

    SERVE_MODES = {"batched": 0, "plain": 1, "overlap": 2}

    def serve(self, handles: list, requests: list[tuple], max_batch: int, budget_bytes: int, mode,
              colors: list[np.ndarray], lanes: int = 7) -> tuple[np.ndarray, np.ndarray, dict]:
        """Runs the native serving loop (sftx_serve) over requests
        [(arrival_s, scene index, frame, samples, max point lights, device bytes)], sorted by
        arrival, in mode "overlap" (continuous batching over submission lanes), "batched" (one
        batch at a time) or "plain" (one request at a time; True and False select "plain" and
        "batched").  colors is the ring of host colour buffers (at least max_batch, each as large
        as the largest request; in "overlap", at most `lanes` batches are in flight).  Returns
        (completion times in s, batch index per request, stats)."""
        if isinstance(mode, bool):
            mode = "plain" if mode else "batched"
        n = len(requests)
        reqs = (SftxRequest * max(1, n))()
        for k, (t, si, f, S, nl, nb) in enumerate(requests):
            reqs[k] = SftxRequest(int(t * 1e9), int(nb), si, f, S, nl)
        hs = (C.c_void_p * len(handles))(*handles)
        cp = (C.c_void_p * len(colors))(*[c.ctypes.data for c in colors])
        done = np.zeros(max(1, n), np.uint64)
        batch = np.zeros(max(1, n), np.uint32)
        st = SftxServeStats()
        rc = self.lib.sftx_serve_ex(hs, reqs, n, max_batch, budget_bytes, self.SERVE_MODES[mode], lanes, cp, len(colors), _ptr(done),
                                 _ptr(batch), C.byref(st))
        self.lib.sft_set_msaa_samples(self.samples)
        if rc != 0:
            raise RuntimeError(f"serving loop failed ({rc}): " + (self.lib.sft_get_last_error() or b"").decode())
        stats = {"batches": st.batches, "max_batch": st.max_batch, "peak_bytes": st.peak_bytes, "max_inflight": st.max_inflight}
        return done[:n].astype(np.float64) * 1e-9, batch[:n].copy(), stats

    def serve_warm(self, handles: list, requests: list[tuple], max_batch: int, budget_bytes: int,
                   colors: list[np.ndarray], lanes: int = 7) -> None:
        """Grows every submission lane (1..lanes, and lane 0) to the largest batch admission can
        form from requests (sftx_serve_warm), so that a serving run that follows allocates
        nothing while it is timed.  Same request tuples and colour ring as serve."""
        n = len(requests)
        reqs = (SftxRequest * max(1, n))()
        for k, (t, si, f, S, nl, nb) in enumerate(requests):
            reqs[k] = SftxRequest(int(t * 1e9), int(nb), si, f, S, nl)
        hs = (C.c_void_p * len(handles))(*handles)
        cp = (C.c_void_p * len(colors))(*[c.ctypes.data for c in colors])
        rc = self.lib.sftx_serve_warm(hs, reqs, n, max_batch, budget_bytes, lanes, cp, len(colors))
        self.lib.sft_set_msaa_samples(self.samples)
        if rc != 0:
            raise RuntimeError(f"serving warm-up failed ({rc}): " + (self.lib.sft_get_last_error() or b"").decode())

    def skeleton_upload(self, rig: dict) -> int:
        """Uploads a rig (scenes.pose_rig layout) with sftg_skeleton_upload; returns its index."""
        ctx = self.lib.sft_get_gpu_context()
        nb = len(rig["bones"])
        bones = (SftgBoneDesc * nb)()
        for i, bd in enumerate(rig["bones"]):
            bones[i].inverse_bind[:] = [float(x) for x in np.asarray(bd["inverse_bind"], np.float32).reshape(-1)]
            bones[i].local_bind[:] = [float(x) for x in np.asarray(bd["local_bind"], np.float32).reshape(-1)]
            bones[i].parent = bd["parent"]
            bones[i].base_t[:] = [float(x) for x in bd["base_t"]]
            bones[i].base_r[:] = [float(x) for x in bd["base_r"]]
            bones[i].base_s[:] = [float(x) for x in bd["base_s"]]
        keep = []   # arrays that must outlive the call
        anims = (SftgAnimationDesc * max(1, len(rig["anims"])))()
        for a, an in enumerate(rig["anims"]):
            smp = (SftgSamplerDesc * len(an["samplers"]))()
            for k, (ins, outs, step) in enumerate(an["samplers"]):
                i_arr = np.ascontiguousarray(ins, np.float32); o_arr = np.ascontiguousarray(outs, np.float32)
                keep += [i_arr, o_arr]
                smp[k] = SftgSamplerDesc(i_arr.ctypes.data, o_arr.ctypes.data, len(i_arr), int(step))
            chs = (SftgChannelDesc * max(1, len(an["channels"])))(*[SftgChannelDesc(*c) for c in an["channels"]])
            keep += [smp, chs]
            anims[a] = SftgAnimationDesc(C.cast(smp, C.c_void_p), C.cast(chs, C.c_void_p), len(an["samplers"]),
                                         len(an["channels"]), float(an["duration"]))
        out = C.c_int32(-1)
        rc = self.lib.sftg_skeleton_upload(ctx, bones, nb, anims, len(rig["anims"]), C.byref(out))
        if rc != 0:
            raise RuntimeError("skeleton upload failed: " + (self.lib.sftg_last_error(ctx) or b"").decode())
        return out.value

    def pose_eval(self, requests: list[tuple[int, int, float]], bone_counts: list[int]) -> tuple[np.ndarray, np.ndarray]:
        """Evaluates [(skeleton, animation, time)] in one sftg_pose_eval; returns (posed, global)
        as flat float32 arrays, request k at offset 16 * sum(bone_counts[:k])."""
        ctx = self.lib.sft_get_gpu_context()
        n = len(requests)
        reqs = (SftgPoseRequest * max(1, n))(*[SftgPoseRequest(s, a, float(t)) for s, a, t in requests])
        total = sum(bone_counts)
        posed = np.zeros(total * 16, np.float32)
        glob = np.zeros(total * 16, np.float32)
        rc = self.lib.sftg_pose_eval(ctx, reqs, n, _ptr(posed), _ptr(glob))
        if rc != 0:
            raise RuntimeError("pose evaluation failed: " + (self.lib.sftg_last_error(ctx) or b"").decode())
        return posed, glob

    def pose_eval_host(self, requests: np.ndarray, posed: np.ndarray, glob: np.ndarray | None = None) -> None:
        """sftg_pose_eval on host arrays: POSE_REQUEST_DTYPE records in, float32 matrices out
        (request k at 16 * the bone counts before it)."""
        ctx = self.lib.sft_get_gpu_context()
        r = np.ascontiguousarray(requests, POSE_REQUEST_DTYPE)
        rc = self.lib.sftg_pose_eval(ctx, r.ctypes.data_as(C.c_void_p), len(r), posed.ctypes.data_as(C.c_void_p),
                                     glob.ctypes.data_as(C.c_void_p) if glob is not None else None)
        if rc != 0:
            raise RuntimeError("pose evaluation failed: " + (self.lib.sftg_last_error(ctx) or b"").decode())

    def pose_eval_device(self, d_requests: int, d_off: int, n: int, d_posed: int, d_global: int = 0) -> None:
        """sftg_pose_eval_device on device pointers (SftgPoseRequest records, u32 offsets in
        matrices, float outputs); asynchronous on the renderer's stream."""
        ctx = self.lib.sft_get_gpu_context()
        rc = self.lib.sftg_pose_eval_device(ctx, C.c_void_p(d_requests), C.c_void_p(d_off), n, C.c_void_p(d_posed),
                                            C.c_void_p(d_global) if d_global else None)
        if rc != 0:
            raise RuntimeError("pose evaluation failed: " + (self.lib.sftg_last_error(ctx) or b"").decode())

    def raycast(self, h, rays: np.ndarray) -> np.ndarray:
        """sft_raycast_batch over RAY_DTYPE records whose `model` indexes the models of scene h
        (one sft_instance per ray with that model and transform); HIT_DTYPE records."""
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        n = len(r)
        insts = (SftInstance * max(1, n))()
        ptrs = (C.c_void_p * max(1, n))()
        models = {}
        for k in range(n):
            mi = int(r[k]["model"])
            if mi not in models:
                models[mi] = self.lib.sftx_scene_model(h, mi)
                if not models[mi]:
                    raise ValueError(f"scene has no model {mi}")
            insts[k].model = models[mi]
            C.memmove(insts[k].transform, r[k]["T"].ctypes.data, 64)
            ptrs[k] = C.addressof(insts[k])
        o = np.ascontiguousarray(r["o"], np.float32)
        d = np.ascontiguousarray(r["d"], np.float32)
        md = np.ascontiguousarray(r["max_dist"], np.float32)
        hits = (SftRayHit * max(1, n))()
        self.lib.sft_raycast_batch(ptrs, _ptr(o), _ptr(d), _ptr(md), n, hits)
        out = np.zeros(n, HIT_DTYPE)
        for k in range(n):
            out[k] = (hits[k].hit, hits[k].distance, tuple(hits[k].pos), tuple(hits[k].normal))
        return out

    def model_device_id(self, h, mi: int) -> int:
        """The resident model id (sftg_model_upload) of model mi of scene h: sft_model's first field."""
        p = self.lib.sftx_scene_model(h, mi)
        if not p:
            raise ValueError(f"scene has no model {mi}")
        return C.c_int32.from_address(p).value

    def last_blas_build(self) -> dict:
        """The last BLAS built on the device at model creation: wall and stream-event ms,
        triangles, kernels launched."""
        w, s, n, k = C.c_double(0), C.c_double(0), C.c_uint32(0), C.c_uint32(0)
        self.lib.sftg_last_blas_build(self.lib.sft_get_gpu_context(), C.byref(w), C.byref(s), C.byref(n), C.byref(k))
        return {"wall_ms": w.value, "stream_ms": s.value, "triangles": n.value, "launches": k.value}

    def model_blas(self, h, mi: int) -> tuple[bytes, int]:
        """(node images, root index) of model mi of scene h through sft_model_get_blas: the BLAS
        the device built at model creation, read back."""
        p = self.lib.sftx_scene_model(h, mi)
        if not p:
            raise ValueError(f"scene has no model {mi}")
        n, root = C.c_uint32(0), C.c_uint32(0)
        nodes = self.lib.sft_model_get_blas(p, C.byref(n), C.byref(root))
        if n.value and not nodes:
            raise RuntimeError("BLAS read-back failed: " + (self.lib.sft_get_last_error() or b"").decode())
        return (C.string_at(nodes, n.value * 256) if n.value else b""), int(root.value)

    def raycast_host(self, rays: np.ndarray, out: np.ndarray | None = None) -> np.ndarray:
        """sftg_raycast on host arrays of RAY_DTYPE records whose `model` is a resident model id;
        hits go to `out` (HIT_DTYPE) when given."""
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        if out is None:
            out = np.zeros(len(r), HIT_DTYPE)
        ctx = self.lib.sft_get_gpu_context()
        if self.lib.sftg_raycast(ctx, _ptr(r), len(r), _ptr(out)) != 0:
            raise RuntimeError("raycast failed: " + (self.lib.sftg_last_error(ctx) or b"").decode())
        return out

    def raycast_device(self, d_rays: int, n: int, d_hits: int) -> None:
        """sftg_raycast_device on device arrays of sftg_ray / sftg_ray_hit (raw pointers), queued
        on the library's stream."""
        ctx = self.lib.sft_get_gpu_context()
        if self.lib.sftg_raycast_device(ctx, C.c_void_p(d_rays), n, C.c_void_p(d_hits)) != 0:
            raise RuntimeError("raycast failed: " + (self.lib.sftg_last_error(ctx) or b"").decode())

    def render_debug(self, h, frame: int, total_ss: int, n_proxies: int, payload_cap: int = 1 << 22,
                     clip_cap: int = 1 << 16) -> dict:
        """Renders one frame and returns the parity buffers named like the oracle's dump sections."""
        w, hh = self.frame_size(h, frame)
        tiles = ((w + 63) // 64) * ((hh + 63) // 64)
        S = self.samples
        out = {
            "depth": np.zeros(tiles * S * 4096, np.float32), "vid": np.zeros(tiles * S * 4096, np.uint32),
            "tile_counts": np.zeros(tiles, np.int32), "tile_payloads_buf": np.zeros(payload_cap, np.uint64),
            "ss_cache": np.zeros(max(1, total_ss) * 576, np.float32), "light_vis": np.zeros(max(1, n_proxies) * 64, np.uint8),
            "clip_buf": np.zeros(clip_cap * 41, np.uint32), "shadow": np.zeros(w * hh * 16 if S == 1 else 1, np.float32),
        }
        pay_total, clip_total, status = np.zeros(1, np.uint64), np.zeros(1, np.uint64), np.zeros(1, np.uint32)
        dbg = SftgDebugOut(_ptr(out["depth"]), _ptr(out["vid"]), _ptr(out["tile_counts"]), _ptr(out["tile_payloads_buf"]),
                           payload_cap, _ptr(pay_total), _ptr(out["ss_cache"]), _ptr(out["light_vis"]), _ptr(out["clip_buf"]),
                           clip_cap, _ptr(clip_total), _ptr(out["shadow"]) if S == 1 else None, _ptr(status))
        self.lib.sft_set_debug_capture(C.byref(dbg))
        try:
            out["color"] = self.render(h, frame).reshape(-1)
        finally:
            self.lib.sft_set_debug_capture(None)
        out["tile_payloads"] = out.pop("tile_payloads_buf")[: int(pay_total[0])].copy()
        out["clip"] = out.pop("clip_buf")[: int(clip_total[0]) * 41].view(np.float32).copy()
        out["ss_cache"] = out["ss_cache"][: total_ss * 576]
        out["light_vis"] = out["light_vis"][: n_proxies * 64]
        out["status"] = int(status[0])
        timings = np.zeros(5, np.float32)
        self.lib.sft_get_frame_timings(_ptr(timings))
        out["timings_ms"] = timings
        return out


def scene_counts(scene, frame: int = 0) -> tuple[int, int]:
    """(screen-space meshlets, world shadow proxies) of a frame of a scenes.Scene."""
    f = scene.frames[frame]
    total_ss = sum(sum(ms.n for ms in scene.models[mi].meshes) for mi, _, _ in f.instances)
    n_prox = sum(len(scene.models[mi].proxies) for mi, _, _ in f.instances) if f.shadows else 0
    return total_ss, n_prox
