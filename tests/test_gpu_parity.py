"""GPU parity: the CUDA render path through the C ABI against the reference's golden digests
(bit-exact visibility buffer, depth, tile lists, screen-space cache, clipped triangles, light
visibility and colour) and against the CPU oracle on fresh seeds."""
import numpy as np
import pytest

import golden_cases as gc
from compare import compare_frames, first_vid_mismatch
from oracle_lib import Oracle
from sofren2_gb300 import runtime, scenes

pytestmark = pytest.mark.gpu


def _render_case(renderer, name, S):
    sc = gc.scene(name)
    h = renderer.load_scene(gc.blob(name))
    try:
        renderer.set_samples(S)
        tss, npx = runtime.scene_counts(sc)
        return renderer.render_debug(h, 0, tss, npx, payload_cap=1 << 23, clip_cap=1 << 16)
    finally:
        renderer.free_scene(h)


@pytest.mark.parametrize("name", list(gc.CASES))
def test_gpu_matches_reference_digests(renderer, golden, name):
    assert gc.sha(memoryview(gc.blob(name))) == golden[name]["scene_sha256"], "scene bytes differ on this platform"
    for S in gc.SAMPLES[name]:
        g = golden[name]["samples"][str(S)]
        out = _render_case(renderer, name, S)
        assert out["status"] == 0
        d, _ = gc.digests(out, g["live_meshlets"], g["clip_used"], gc.n_lights(name))
        mism = [k for k in d if k in g and d[k] != g[k]]
        assert not mism, f"{name} {S}x differs from the reference in {mism}"


@pytest.mark.parametrize("seed", [21, 22, 23, 24])
@pytest.mark.parametrize("samples", [1, 2, 4])
def test_gpu_equals_oracle_random(renderer, seed, samples):
    kind = seed % 3
    if kind == 0:
        sc = scenes.variety_scene(width=256, height=160, seed=seed, n_objects=16, n_lights=4 + seed % 15)
    elif kind == 1:
        sc = scenes.skinned_characters_scene(320, 192, seed=seed, n_chars=3, tex_size=32, ground_quads=12)
    else:
        sc = scenes.static_shapes_scene(300, 170, seed=seed, n_spheres=5, n_cubes=5, tex_size=32)
    blob = sc.to_bytes()
    o = Oracle(blob)
    try:
        ref = o.render_dump(0, samples)
    finally:
        o.close()
    assert ref["invalid_packets"] == 0
    h = renderer.load_scene(blob)
    try:
        renderer.set_samples(samples)
        tss, npx = runtime.scene_counts(sc)
        out = renderer.render_debug(h, 0, tss, npx)
    finally:
        renderer.free_scene(h)
    res = compare_frames(ref, out, samples, len(sc.frames[0].point_lights))
    bad = {k: v for k, v in res.items() if k not in ("color_max_lsb", "tlas") and v != 0}
    cols = (sc.frames[0].width + 63) // 64
    assert not bad, (res, first_vid_mismatch(ref, out, cols, samples))


@pytest.mark.parametrize("seed", [31, 32])
@pytest.mark.parametrize("samples", [1, 4])
def test_gpu_equals_oracle_random_atrium(renderer, seed, samples):
    """Fresh seeds of the lightmapped atrium (pillars, arches, lightmap pages, skinned humanoids,
    10 point lights) at a small size: the lightmap shading path against the oracle."""
    sc = scenes.atrium_scene(width=256, height=160, seed=seed, nx=6, nz=4, levels=2, arch_segments=6, n_tex=4, tex_size=64,
                             lm_size=128, n_lights=10, n_chars=2, char_tex=64, floor_quads=(24, 12))
    blob = sc.to_bytes()
    o = Oracle(blob)
    try:
        ref = o.render_dump(0, samples)
    finally:
        o.close()
    assert ref["invalid_packets"] == 0
    h = renderer.load_scene(blob)
    try:
        renderer.set_samples(samples)
        tss, npx = runtime.scene_counts(sc)
        out = renderer.render_debug(h, 0, tss, npx)
    finally:
        renderer.free_scene(h)
    res = compare_frames(ref, out, samples, len(sc.frames[0].point_lights))
    bad = {k: v for k, v in res.items() if k not in ("color_max_lsb", "tlas") and v != 0}
    cols = (sc.frames[0].width + 63) // 64
    assert not bad, (res, first_vid_mismatch(ref, out, cols, samples))


def test_gpu_shadow_factors_equal_oracle(renderer):
    """Per-pixel shadow intensity of every tile light (1x) is identical to the FP32 oracle
    (the tolerance stated for shadow factors is 1e-5 absolute).  The FP32 values against an FP64
    evaluation of the same expression are measured on the CPU in test_shadow_fp64.py."""
    sc = gc.scene("skinned_small")
    blob = gc.blob("skinned_small")
    w, h_ = sc.frames[0].width, sc.frames[0].height
    o = Oracle(blob)
    try:
        _, _, sh_o = o.render_color(0, 1, w, h_, shadow=True)
    finally:
        o.close()
    h = renderer.load_scene(blob)
    try:
        renderer.set_samples(1)
        tss, npx = runtime.scene_counts(sc)
        out = renderer.render_debug(h, 0, tss, npx)
    finally:
        renderer.free_scene(h)
    sg = out["shadow"]
    assert np.array_equal(sg.view(np.uint32), sh_o.view(np.uint32))
    assert float(np.max(np.abs(sg - sh_o))) <= 1e-5


def test_api_pitch_and_host_buffer(renderer):
    """The caller's colour buffer is written through its pitch and nothing else is touched."""
    name = "small"
    sc = gc.scene(name)
    w, hh = sc.frames[0].width, sc.frames[0].height
    h = renderer.load_scene(gc.blob(name))
    try:
        renderer.set_samples(1)
        tight = renderer.render(h, 0)
        padded = np.full((hh, w + 13), 0xDEADBEEF, dtype=np.uint32)
        renderer.render(h, 0, padded)
    finally:
        renderer.free_scene(h)
    assert np.array_equal(padded[:, :w], tight)
    assert np.all(padded[:, w:] == 0xDEADBEEF)
