"""Colour written in place into a page-locked caller buffer (the resolve stores straight to host
memory, no device-to-host copy): the same pixels as the copy path through a pageable buffer and
as the reference's digests, also with a row pitch wider than the frame, in a batch with pageable
views beside it, and with the keep-the-caller's-pixels mode (which stays on the copy path)."""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

CASES = ["small", "config1", "skinned_small", "atrium_small", "variety_noclear"]


def _pinned(h, w, pad):
    torch = pytest.importorskip("torch")
    t = torch.zeros((h, w + pad), dtype=torch.int32).pin_memory()
    return t, t.numpy().view(np.uint32)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("pad", [0, 24])
def test_pinned_buffer_matches_copy_path(renderer, golden, name, pad):
    h = renderer.load_scene(gc.blob(name))
    try:
        for S in gc.SAMPLES[name]:
            renderer.set_samples(S)
            w, hh = renderer.frame_size(h, 0)
            init = np.random.default_rng(S + pad).integers(0, 1 << 32, size=(hh, w), dtype=np.uint32)
            ref = renderer.render(h, 0, init.copy())
            keep, buf = _pinned(hh, w, pad)
            buf[:, :w] = init
            got = renderer.render(h, 0, buf[:, :w])
            assert np.array_equal(got, ref), f"{name} {S}x: pinned buffer differs from the copy path"
            if pad:
                assert not buf[:, w:].any(), "pixels written past the frame width"
            if name != "variety_noclear":
                assert gc.sha(np.ascontiguousarray(got).reshape(-1)) == golden[name]["samples"][str(S)]["color"]
    finally:
        renderer.set_samples(1)
        renderer.free_scene(h)


def test_pinned_and_pageable_views_in_one_batch(renderer):
    names = ["small", "skinned_small", "atrium_small", "config1"]
    hs = [renderer.load_scene(gc.blob(n)) for n in names]
    try:
        views = [(h, 0, S) for h in hs for S in (1, 4)]
        alone = []
        for hh_, f, S in views:
            renderer.set_samples(S)
            alone.append(renderer.render(hh_, f))
        renderer.set_samples(1)
        colors, keep = [], []
        for k, (hh_, f, S) in enumerate(views):
            w, h = renderer.frame_size(hh_, f)
            if k % 2:
                t, b = _pinned(h, w, 8)
                keep.append(t)
                colors.append(b[:, :w])
            else:
                colors.append(np.zeros((h, w), np.uint32))
        got = renderer.render_batch(views, colors)
        for k, (a, b) in enumerate(zip(alone, got)):
            assert np.array_equal(a, b), f"view {k} ({'pinned' if k % 2 else 'pageable'}) differs from its lone render"
    finally:
        for h in hs:
            renderer.free_scene(h)


@pytest.mark.parametrize("mode", [1, 2, 3, 4, 5])
def test_debug_views_into_pinned_buffer(renderer, mode):
    """The debug views (the overlays read and blend the colour in place) give the same pixels
    in a page-locked buffer with a padded pitch as through the copy path."""
    h = renderer.load_scene(gc.blob("variety"))
    try:
        renderer.set_debug_mode(mode)
        for S in (1, 4):
            renderer.set_samples(S)
            w, hh = renderer.frame_size(h, 0)
            ref = renderer.render(h, 0)
            keep, buf = _pinned(hh, w, 16)
            got = renderer.render(h, 0, buf[:, :w])
            assert np.array_equal(got, ref), f"debug view {mode} at {S}x differs in a pinned buffer"
    finally:
        renderer.set_debug_mode(0)
        renderer.set_samples(1)
        renderer.free_scene(h)
