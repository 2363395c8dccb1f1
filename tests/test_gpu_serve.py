"""Served rendering (sftx_serve, the native serving loop): every request's pixels are the ones a
lone render of it produces, whether it was served with batches overlapping on the GPU (overlap,
continuous batching over submission lanes), one batch at a time, alone (plain) or under a memory
budget that forces one request per batch; and batches queued on different submission lanes
(sft_batch_submit_async) without waiting in between give every view its lone pixels."""
import ctypes as C

import numpy as np
import pytest

from sofren2_gb300 import runtime, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(renderer):
    scs, samples = scenes.config5(n_scenes=4, frames_per_scene=3, quick=True)
    hs = [renderer.load_scene(sc.to_bytes()) for sc in scs]
    rng = np.random.default_rng(5)
    reqs = []
    for k in range(24):
        si = int(rng.integers(len(scs)))
        f = int(rng.integers(3))
        fr = scs[si].frames[f]
        meshlets = sum(sum(ms.n for ms in scs[si].models[mi].meshes) for mi, _, _ in fr.instances)
        nb = runtime.request_device_bytes(fr.width, fr.height, samples[si], meshlets)
        reqs.append((0.0005 * (k // 6), si, f, samples[si], int(rng.integers(1, 17)), nb))
    sizes = [(scs[si].frames[f].width, scs[si].frames[f].height) for _, si, f, _, _, _ in reqs]
    alone = []
    for (_, si, f, S, nl, _), (w, h) in zip(reqs, sizes):
        renderer.set_samples(S)
        c = np.zeros((h, w), np.uint32)
        assert renderer.lib.sftx_scene_render_ex(hs[si], f, c.ctypes.data, c.strides[0], nl) == 0
        alone.append(c)
    renderer.set_samples(1)
    yield hs, reqs, sizes, alone
    for h in hs:
        renderer.free_scene(h)


def _ring(sizes, n):
    big = max(w * h for w, h in sizes)
    return [np.zeros(big, np.uint32) for _ in range(n)]


def _check(colors, sizes, alone):
    for k, ((w, h), a) in enumerate(zip(sizes, alone)):
        got = colors[k][: w * h].reshape(h, w)
        assert np.array_equal(got, a), f"request {k} differs from its lone render"


@pytest.mark.parametrize("mode", ["overlap", "batched", "plain"])
def test_served_equals_alone(renderer, served, mode):
    hs, reqs, sizes, alone = served
    colors = _ring(sizes, len(reqs))
    done, batch, st = renderer.serve(hs, reqs, max_batch=8, budget_bytes=1 << 40, mode=mode, colors=colors)
    _check(colors, sizes, alone)
    assert np.all(done >= np.array([r[0] for r in reqs]))
    if mode == "plain":
        assert st["max_batch"] == 1 and st["batches"] == len(reqs)
    else:
        assert 1 < st["max_batch"] <= 8 and st["batches"] < len(reqs)
    if mode == "overlap":
        assert 1 <= st["max_inflight"] <= 7


def test_warm_then_serve(renderer, served):
    """The warm-up renders the largest batch on every lane (the requests with the largest device
    estimates, largest first, into the ring's first slots), then a served run over the grown lanes
    still gives every request its lone pixels."""
    hs, reqs, sizes, alone = served
    colors = _ring(sizes, len(reqs))
    renderer.serve_warm(hs, reqs, max_batch=5, budget_bytes=1 << 40, colors=colors, lanes=7)
    order = sorted(range(len(reqs)), key=lambda k: (-reqs[k][5], k))[:5]
    for slot, k in enumerate(order):
        w, h = sizes[k]
        assert np.array_equal(colors[slot][: w * h].reshape(h, w), alone[k]), f"warm-up slot {slot} (request {k})"
    colors = _ring(sizes, len(reqs))
    renderer.serve(hs, reqs, max_batch=8, budget_bytes=1 << 40, mode="overlap", colors=colors)
    _check(colors, sizes, alone)


def test_overlap_with_a_small_colour_ring(renderer, served):
    """8 colour buffers for 24 requests: a ring slot is handed out again only after its request
    has finished, so the last 8 requests' slots hold their lone pixels."""
    hs, reqs, sizes, alone = served
    colors = _ring(sizes, 8)
    done, batch, st = renderer.serve(hs, reqs, max_batch=4, budget_bytes=1 << 40, mode="overlap", colors=colors)
    n = len(reqs)
    for k in range(n - 8, n):
        w, h = sizes[k]
        assert np.array_equal(colors[k % 8][: w * h].reshape(h, w), alone[k]), f"request {k} differs from its lone render"


def test_batches_on_lanes_overlap(renderer, served):
    hs, reqs, sizes, alone = served
    lib = renderer.lib
    colors = _ring(sizes, len(reqs))
    groups = [list(range(0, 8)), list(range(8, 14)), list(range(14, 24))]
    for lane, g in zip((1, 2, 3), groups):   # three batches queued before any is waited for
        lib.sft_batch_begin()
        for k in g:
            _, si, f, S, nl, _ = reqs[k]
            renderer.set_samples(S)
            assert lib.sftx_scene_render_ex(hs[si], f, colors[k].ctypes.data, 0, nl) == 0
        assert lib.sft_batch_submit_async(lane) == 0
    renderer.set_samples(1)
    for lane in (3, 1, 2):
        assert lib.sft_batch_wait(lane) == 0
        assert lib.sft_batch_done(lane) == 1
    _check(colors, sizes, alone)


def test_memory_budget_limits_batches(renderer, served):
    hs, reqs, sizes, alone = served
    colors = _ring(sizes, len(reqs))
    budget = min(r[5] for r in reqs)   # any two requests exceed it: one request per batch
    done, batch, st = renderer.serve(hs, reqs, max_batch=8, budget_bytes=budget, mode="batched", colors=colors)
    _check(colors, sizes, alone)
    assert st["max_batch"] == 1


def test_memory_budget_limits_overlapping_batches(renderer, served):
    hs, reqs, sizes, alone = served
    colors = _ring(sizes, len(reqs))
    budget = min(r[5] for r in reqs)   # one request in flight at a time over all lanes
    done, batch, st = renderer.serve(hs, reqs, max_batch=8, budget_bytes=budget, mode="overlap", colors=colors)
    _check(colors, sizes, alone)
    assert st["max_batch"] == 1 and st["max_inflight"] == 1


def test_lane_submission_errors(renderer, served):
    """sftg_frames_submit refuses lane 0 (the synchronous lane), lanes past the last and a lane
    with a batch in flight; the batch in flight then finishes normally."""
    hs, reqs, sizes, alone = served
    lib = renderer.lib
    lib.sft_batch_peek.restype = C.c_void_p
    lib.sft_batch_peek.argtypes = [C.c_uint32]
    lib.sftg_frames_submit.restype = C.c_int
    lib.sftg_frames_submit.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    lib.sftg_lane_done.restype = C.c_int
    lib.sftg_lane_done.argtypes = [C.c_void_p, C.c_uint32]
    lib.sftg_lane_wait.restype = C.c_int
    lib.sftg_lane_wait.argtypes = [C.c_void_p, C.c_uint32]
    ctx = lib.sft_get_gpu_context()
    _, si, f, S, nl, _ = reqs[0]
    lib.sft_batch_begin()
    renderer.set_samples(S)
    assert lib.sftx_scene_render_ex(hs[si], f, None, 0, nl) == 0
    desc = lib.sft_batch_peek(0)
    assert desc
    assert lib.sftg_frames_submit(ctx, 0, desc, 1, None, None) == -2
    assert lib.sftg_frames_submit(ctx, 8, desc, 1, None, None) == -2
    assert lib.sftg_frames_submit(ctx, 1, desc, 1, None, None) == 0
    assert lib.sftg_frames_submit(ctx, 1, desc, 1, None, None) == -2   # busy
    assert lib.sftg_lane_done(ctx, 1) in (0, 1)
    assert lib.sftg_lane_wait(ctx, 1) == 0
    assert lib.sftg_lane_done(ctx, 1) == 1
    assert lib.sft_batch_submit() == 0   # the recorded frame, rendered on the synchronous lane
    renderer.set_samples(1)


def test_overlap_into_pinned_buffers(renderer, served):
    """Batches in flight on several lanes, each writing its frames straight into page-locked
    request buffers: every request still gets its lone pixels."""
    torch = pytest.importorskip("torch")
    hs, reqs, sizes, alone = served
    big = max(w * h for w, h in sizes)
    keep = [torch.zeros(big, dtype=torch.int32).pin_memory() for _ in reqs]
    colors = [t.numpy().view(np.uint32) for t in keep]
    done, batch, st = renderer.serve(hs, reqs, max_batch=4, budget_bytes=1 << 40, mode="overlap", colors=colors)
    _check(colors, sizes, alone)
