"""Batched submission (sftg_frames_render through sft_batch_begin / sft_batch_submit): every view
of a mixed batch (different scenes, sizes, sample counts, clear and keep-the-caller's-pixels
modes) equals the same view rendered alone, pixel for pixel, and the golden cases rendered
together in one batch still match the reference's colour digests."""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

MIXED = ["small", "skinned_small", "atrium_small", "variety", "variety_noclear", "config1"]


def _initial(renderer, h, f, seed):
    w, hh = renderer.frame_size(h, f)
    return np.random.default_rng(seed).integers(0, 1 << 32, size=(hh, w), dtype=np.uint32)


def _alone(renderer, views, inits):
    out = []
    for (h, f, S), init in zip(views, inits):
        renderer.set_samples(S)
        out.append(renderer.render(h, f, init.copy()))
    renderer.set_samples(1)
    return out


@pytest.fixture(scope="module")
def handles(renderer):
    hs = {n: renderer.load_scene(gc.blob(n)) for n in MIXED}
    yield hs
    for h in hs.values():
        renderer.free_scene(h)


def test_batch_equals_single_views(renderer, handles):
    views = [(handles[n], 0, S) for S in (4, 1, 2) for n in MIXED]
    inits = [_initial(renderer, h, f, 100 + i) for i, (h, f, _) in enumerate(views)]
    alone = _alone(renderer, views, inits)
    got = renderer.render_batch(views, [i.copy() for i in inits])
    for k, (a, b) in enumerate(zip(alone, got)):
        bad = int(np.count_nonzero(a != b))
        assert bad == 0, f"view {k} ({MIXED[k % len(MIXED)]}, {views[k][2]}x): {bad} pixels differ from the single-view render"


def test_batch_repeat_and_order(renderer, handles):
    """The same views in another order, twice in a row, and a one-view batch."""
    views = [(handles[n], 0, S) for n, S in zip(MIXED, (1, 2, 4, 2, 1, 4))]
    inits = [_initial(renderer, h, f, 200 + i) for i, (h, f, _) in enumerate(views)]
    alone = _alone(renderer, views, inits)
    order = [5, 0, 3, 1, 4, 2]
    for _ in range(2):
        got = renderer.render_batch([views[k] for k in order], [inits[k].copy() for k in order])
        for j, k in enumerate(order):
            assert np.array_equal(got[j], alone[k]), f"view {k} differs in the reordered batch"
    one = renderer.render_batch([views[2]], [inits[2].copy()])
    assert np.array_equal(one[0], alone[2])


def test_batch_device_only_then_host(renderer, handles):
    """A device-only batch (no host colour buffers) followed by a host batch gives the same pixels."""
    views = [(handles[n], 0, 2) for n in MIXED if n != "variety_noclear"]
    renderer.render_batch(views, None)
    got = renderer.render_batch(views, [None] * len(views))
    alone = _alone(renderer, views, [np.zeros_like(g) for g in got])
    for a, b in zip(alone, got):
        assert np.array_equal(a, b)


def test_golden_cases_in_one_batch(renderer, golden):
    names = [n for n in gc.CASES if n != "variety_noclear"]
    hs = [renderer.load_scene(gc.blob(n)) for n in names]
    try:
        views, keys = [], []
        for n, h in zip(names, hs):
            for S in gc.SAMPLES[n]:
                views.append((h, 0, S))
                keys.append((n, S))
        got = renderer.render_batch(views, [None] * len(views))
        for (n, S), c in zip(keys, got):
            assert gc.sha(c.reshape(-1)) == golden[n]["samples"][str(S)]["color"], f"{n} {S}x colour differs inside a batch"
    finally:
        for h in hs:
            renderer.free_scene(h)


TUNINGS = [
    dict(resolve_split=(1, 2, 8), raster_slab_rows=(4, 16, 64), geom_job_width=1, raster_bands=(1, 2, 4), tile_lights=(2, 1, 2)),
    dict(resolve_split=(8, 1, 2), raster_slab_rows=(64, 4, 16), geom_job_width=3, raster_bands=(4, 1, 2), tile_lights=(1, 2, 1),
         tile_queue=3),
    dict(resolve_split=(2, 8, 1), raster_slab_rows=(16, 64, 4), geom_job_width=5, raster_bands=(2, 4, 1), tile_lights=(2, 2, 2)),
    dict(resolve_split=(16, 16, 16), raster_slab_rows=(4, 4, 4), geom_job_width=8, tile_lights=(1, 1, 1), tile_queue=1),
    dict(resolve_split=(4, 4, 4), raster_slab_rows=(8, 8, 8), geom_job_width=2, tile_lights=(2, 2, 1), tile_queue=2),
    dict(resolve_split=(16, 8, 16), raster_slab_rows=(8, 8, 4), geom_job_width=8, occl_ray_prune=1),
]


@pytest.mark.parametrize("tuning", TUNINGS)
def test_tuning_knobs_do_not_change_results(renderer, golden, tuning):
    """Every scheduling knob of sftg_tuning leaves every pixel of every golden case unchanged."""
    names = [n for n in gc.CASES if n != "variety_noclear"]
    hs = [renderer.load_scene(gc.blob(n)) for n in names]
    saved = renderer.tuning()
    try:
        renderer.set_tuning(**tuning)
        views, keys = [], []
        for n, h in zip(names, hs):
            for S in gc.SAMPLES[n]:
                views.append((h, 0, S))
                keys.append((n, S))
        got = renderer.render_batch(views, [None] * len(views))
        for (n, S), c in zip(keys, got):
            assert gc.sha(c.reshape(-1)) == golden[n]["samples"][str(S)]["color"], f"{n} {S}x differs with {tuning}"
    finally:
        renderer.set_tuning(**saved)
        for h in hs:
            renderer.free_scene(h)


def test_autotune_keeps_results(renderer, golden, handles):
    views = [(handles[n], 0, S) for n, S in zip(MIXED, (1, 2, 4, 2, 1, 4)) if n != "variety_noclear"]
    saved = renderer.tuning()
    try:
        t = renderer.autotune_batch(views, reps=1)
        assert t["geom_job_width"] in (1, 2, 4, 8)
        h = renderer.load_scene(gc.blob("config1"))
        try:
            got = renderer.render_batch([(h, 0, 2)], [None])
            assert gc.sha(got[0].reshape(-1)) == golden["config1"]["samples"]["2"]["color"]
        finally:
            renderer.free_scene(h)
    finally:
        renderer.set_tuning(**saved)


@pytest.mark.parametrize("lanes", [2, 3, 7])
def test_batch_split_over_lanes_equals_single_views(renderer, handles, lanes):
    """The mixed views as `lanes` batches overlapping on submission lanes give every view its
    lone pixels, twice in a row (the second time replaying each lane's captured graph)."""
    views = [(handles[n], 0, S) for S in (4, 1, 2) for n in MIXED]
    inits = [_initial(renderer, h, f, 300 + i) for i, (h, f, _) in enumerate(views)]
    alone = _alone(renderer, views, inits)
    for _ in range(2):
        got = renderer.render_batch(views, [i.copy() for i in inits], lanes=lanes)
        for k, (a, b) in enumerate(zip(alone, got)):
            assert np.array_equal(a, b), f"view {k} differs when the batch is split over {lanes} lanes"
