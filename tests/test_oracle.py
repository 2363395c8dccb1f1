"""The CPU oracle against the reference's golden digests, and against the reference itself on
fresh seeds where the reference is compiled here (oracle/_ref, x86-64 only)."""
import numpy as np
import pytest

import golden_cases as gc
from compare import compare_frames
from oracle_lib import Oracle, reference_available, reference_dump


@pytest.mark.parametrize("name", gc.FAST)
def test_scene_bytes_pinned(golden, name):
    assert gc.sha(memoryview(gc.blob(name))) == golden[name]["scene_sha256"]


@pytest.mark.parametrize("name", gc.FAST)
def test_oracle_matches_reference_digests(golden, name):
    o = Oracle(gc.blob(name))
    try:
        for S in gc.SAMPLES[name]:
            g = golden[name]["samples"][str(S)]
            frame = o.render_dump(0, S)
            d, _ = gc.digests(frame, g["live_meshlets"], g["clip_used"], gc.n_lights(name))
            mism = [k for k in d if k in g and d[k] != g[k]]
            assert not mism, f"{name} {S}x: sections differ from the reference: {mism}"
            assert frame["invalid_packets"] == 0
    finally:
        o.close()


@pytest.mark.slow
@pytest.mark.parametrize("name", ["config2", "config3"])
def test_oracle_matches_reference_digests_full(golden, name):
    o = Oracle(gc.blob(name))
    try:
        for S in gc.SAMPLES[name]:
            g = golden[name]["samples"][str(S)]
            d, _ = gc.digests(o.render_dump(0, S, threads=8), g["live_meshlets"], g["clip_used"], gc.n_lights(name))
            assert [k for k in d if k in g and d[k] != g[k]] == []
    finally:
        o.close()


def test_oracle_hand_padding_rows_hold_x86_default_nan(golden):
    """The hand case's meshlets hold 3 live vertices; the 61 padding slots sit at the camera
    position, so w = 0 and rcp_refined(0) = RCPPS(0) * fnmadd(0, inf, 2) is an invalid operation.
    x86 writes its default NaN 0xFFC00000 into sx, sy and inv_w there (sofren2.c:633-638,
    5109-5122); the oracle must write the same bits on any host (aarch64's default NaN is
    0x7FC00000), and no other NaN pattern may appear."""
    o = Oracle(gc.blob("hand"))
    try:
        frame = o.render_dump(0, 1)
    finally:
        o.close()
    g = golden["hand"]["samples"]["1"]
    ss = frame["ss_cache"].view(np.uint32).reshape(-1, 9, 64)[np.asarray(g["live_meshlets"], dtype=np.int64)]
    isnan = (ss & 0x7F800000) == 0x7F800000
    isnan &= (ss & 0x007FFFFF) != 0
    assert np.all(ss[isnan] == 0xFFC00000)
    per_row = isnan.sum(axis=(0, 2))
    assert per_row[0] == per_row[1] == per_row[2] > 0, per_row   # sx, sy, inv_w
    assert per_row[3:].sum() == 0, per_row                        # world position and normal stay finite


SEEDS = [11, 12, 13]


@pytest.mark.skipif(not reference_available(1), reason="reference not compiled here (oracle/_ref, x86-64 with AVX2)")
@pytest.mark.parametrize("seed", SEEDS)
@pytest.mark.parametrize("samples", [1, 2, 4])
def test_oracle_equals_reference_random(seed, samples):
    from sofren2_gb300 import scenes
    sc = scenes.variety_scene(width=192, height=128, seed=seed, n_objects=14, n_lights=6 + seed % 12)
    blob = sc.to_bytes()
    r = reference_dump(blob, samples)[0]
    o = Oracle(blob)
    try:
        g = o.render_dump(0, samples)
    finally:
        o.close()
    res = compare_frames(r, g, samples, len(sc.frames[0].point_lights))
    bad = {k: v for k, v in res.items() if k != "color_max_lsb" and v != 0}
    assert not bad, res


def _skinned(seed):
    from sofren2_gb300 import scenes
    return scenes.skinned_characters_scene(width=256, height=160, seed=seed, n_chars=3, n_lights=6, tex_size=64)


def _atrium(seed):
    from sofren2_gb300 import scenes
    return scenes.atrium_scene(width=256, height=160, seed=seed, nx=6, nz=4, levels=2, arch_segments=6, n_tex=4, tex_size=64,
                               lm_size=128, n_lights=10, n_chars=2, char_tex=64, floor_quads=(24, 12))


@pytest.mark.skipif(not reference_available(1), reason="reference not compiled here (oracle/_ref, x86-64 with AVX2)")
@pytest.mark.parametrize("kind,samples", [("skinned", 2), ("atrium", 4)])
@pytest.mark.parametrize("seed", [31, 32])
def test_oracle_equals_reference_random_workload_shapes(kind, samples, seed):
    """Fresh seeds of the two 1080p workloads' scene families at a small size: skinned humanoids
    with capsule proxies at 2x, and the lightmapped atrium with skinned humanoids at 4x."""
    sc = (_skinned if kind == "skinned" else _atrium)(seed)
    blob = sc.to_bytes()
    r = reference_dump(blob, samples)[0]
    o = Oracle(blob)
    try:
        g = o.render_dump(0, samples)
    finally:
        o.close()
    res = compare_frames(r, g, samples, len(sc.frames[0].point_lights))
    bad = {k: v for k, v in res.items() if k != "color_max_lsb" and v != 0}
    assert not bad, res


def test_oracle_detects_undefined_packet_frustum():
    """A light inside a proxy batch's bounding box leaves the reference's packet frustum
    uninitialised (sofren2.c:4044-4048); the oracle counts those packets so parity scenes can
    exclude them."""
    from sofren2_gb300 import scenes
    sc = scenes.static_shapes_scene(160, 96, seed=9, n_spheres=4, n_cubes=4, tex_size=32)
    lp, *rest = sc.frames[0].point_lights[0]
    sc.frames[0].point_lights = [((np.float32(0.0), np.float32(0.0), np.float32(25.0)), *rest)]
    o = Oracle(sc.to_bytes())
    try:
        assert o.render_dump(0, 1)["invalid_packets"] > 0
    finally:
        o.close()


@pytest.mark.parametrize("case", gc.DEBUG_CASES, ids=lambda c: f"{c[0]}-{c[1]}-{c[2]}x")
def test_oracle_debug_views_match_reference(golden, case):
    """Debug views (wireframe, tile grid, depth, light count, checkerboard) against the
    reference's own renders with sft_set_debug_mode."""
    name, mode, S = case
    sc = gc.scene(name)
    o = Oracle(gc.blob(name))
    try:
        o.set_debug_mode(mode)
        color, _, _ = o.render_color(0, S, sc.frames[0].width, sc.frames[0].height)
    finally:
        o.close()
    assert gc.sha(color) == golden["debug_views"][f"{name}/{mode}/{S}"]


def test_oracle_pose_matches_reference(golden):
    """The oracle's sft_pose_update restatement against the reference's own output on a seeded
    rig: every slerp branch, stepped and linear samplers, wrapped and clamped times, a later
    channel overriding an earlier one, an out-of-range node, out-of-range animations."""
    from oracle_lib import oracle_pose, pose_blob, reference_pose, reference_pose_available
    from sofren2_gb300 import scenes
    rig = scenes.pose_rig()
    req = scenes.pose_requests(rig, golden["pose"]["requests"])
    blob = pose_blob(rig, req)
    o = oracle_pose(blob, len(rig["bones"]), len(req))
    assert gc.sha(o) == golden["pose"]["sha256"]
    if reference_pose_available():
        r = reference_pose(blob, len(rig["bones"]), len(req))
        assert np.array_equal(o.view(np.uint32), r.view(np.uint32))
