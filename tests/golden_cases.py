"""The golden parity cases: seeded scenes rendered by the reference (tests/golden/make_golden.py)
and re-checked against the CPU oracle and the GPU library.  Each case names a scene generator
and its arguments; the scene bytes themselves are regenerated deterministically (their SHA-256
is pinned too, so a platform that generated different bytes fails loudly)."""
from __future__ import annotations

import hashlib

import numpy as np

from sofren2_gb300 import scenes

CASES = {
    "small": ("static_shapes_scene", dict(width=200, height=136, seed=7, n_spheres=3, n_cubes=3, tex_size=64)),
    "config1": ("config1", dict()),
    "skinned_small": ("skinned_characters_scene", dict(width=640, height=360, seed=3, n_chars=4, tex_size=64, ground_quads=16)),
    "atrium_small": ("atrium_scene", dict(width=320, height=200, seed=5, nx=4, nz=3, levels=2, arch_segments=8, n_tex=3,
                                          tex_size=64, lm_size=256, n_lights=5, n_chars=2, char_tex=64, floor_quads=(12, 6))),
    "variety": ("variety_scene", dict()),
    "variety_noclear": ("variety_scene", dict(seed=4002, clear=0)),
    "config2": ("config2", dict()),
    "config3": ("config3", dict()),
    "hand": ("hand_scene", dict()),
}

# cases the CPU oracle re-checks in the default (not-gpu) test run; the big configurations are
# checked on the GPU against their digests, and against the oracle in the slow tier
FAST = ["small", "config1", "skinned_small", "atrium_small", "variety", "variety_noclear", "hand"]
# debug views (enum sft_debug_mode 1..5) over a few cases: (case, mode, samples)
DEBUG_CASES = [(n, m, S) for n in ("small", "variety", "atrium_small") for m in (1, 2, 3, 4, 5) for S in (1, 4)]
SAMPLES = {name: (1, 2, 4) for name in CASES}
SAMPLES["config2"] = (2,)
SAMPLES["config3"] = (4,)

_cache: dict = {}


def hand_scene(width: int = 200, height: int = 136):
    """Hand-made edge cases in one view: a single triangle with a 1x1 texture, a triangle seen
    edge-on (its plane holds the camera), two coplanar triangles sharing an edge with different
    textures (the tie order on the shared edge), two floor triangles crossing the near plane
    with one and with two vertices in front, and 17 point lights clustered so that some tiles
    hold more than the 16-light cap, some one light and some none; a capsule proxy over the
    single triangle casts shadows from the cluster."""
    sc = scenes.Scene()
    one = sc.add_material(sc.add_texture(np.array([[0xFF3080C0]], np.uint32)), 0xFFFFFFFF, 16.0)
    ta = sc.add_material(sc.add_texture(scenes.value_noise_texture(8, 8, 91)), 0xFFFFFFFF, 8.0)
    tb = sc.add_material(sc.add_texture(scenes.value_noise_texture(16, 8, 92, lattice=4)), 0xFFC0A080, 32.0)

    def mesh(pos, nrm, tris):
        pos = np.asarray(pos, np.float32)
        nrm = np.tile(np.asarray(nrm, np.float32), (len(pos), 1))
        uv = np.asarray([[0.1 + 0.8 * (k % 2), 0.1 + 0.4 * (k % 3)] for k in range(len(pos))], np.float32)
        return scenes.build_meshlets(scenes.RawMesh(pos, nrm, uv, scenes._orient(pos, nrm, np.asarray(tris))))

    towards = (0.0, 0.0, -1.0)
    tri = mesh([(-1.2, 0.2, 3.0), (-0.6, 0.2, 3.0), (-0.9, 0.7, 3.0)], towards, [[0, 1, 2]])
    edge = mesh([(0.2, 0.5, 2.0), (0.6, 0.75, 3.0), (0.4, 1.0, 4.0)], (1.0, 0.0, 0.0), [[0, 1, 2]])
    q = [(0.6, -0.8, 2.5), (1.4, -0.8, 2.5), (1.4, -0.1, 2.5), (0.6, -0.1, 2.5)]
    quad_a = mesh([q[0], q[1], q[2]], towards, [[0, 1, 2]])
    quad_b = mesh([q[0], q[2], q[3]], towards, [[0, 1, 2]])
    up = (0.0, 1.0, 0.0)
    near1 = mesh([(-0.5, -0.25, -0.5), (0.5, -0.25, -0.5), (0.0, -0.25, 1.5)], up, [[0, 1, 2]])
    near2 = mesh([(-0.9, -0.35, 1.2), (-0.3, -0.35, 1.2), (-0.6, -0.35, -0.4)], up, [[0, 1, 2]])
    models = [
        sc.add_model(scenes.Model([tri], [one], proxies=[((-1.0, 0.3, 2.7), (-0.8, 0.5, 2.7), 0.08, 0xFFFFFFFF)])),
        sc.add_model(scenes.Model([edge], [ta])),
        sc.add_model(scenes.Model([quad_a, quad_b], [ta, tb])),
        sc.add_model(scenes.Model([near1, near2], [tb, ta])),
    ]
    fr = scenes._camera_frame(width, height)
    for k in range(17):
        a = 2.0 * np.pi * k / 17.0
        fr.point_lights.append(((-0.9 + 0.25 * np.cos(a), 0.45 + 0.25 * np.sin(a), 2.4), 1.0, 0.9, 0.8, 0.1, 0.7))
    fr.point_lights.append(((1.0, -0.45, 2.0), 0.7, 0.8, 1.0, 1.5, 1.0))
    for mi in models:
        fr.instances.append((mi, scenes.mat_identity(), None))
    sc.frames.append(fr)
    return sc


_LOCAL = {"hand_scene": hand_scene}


def scene(name: str):
    if name not in _cache:
        fn, kw = CASES[name]
        _cache[name] = (_LOCAL.get(fn) or getattr(scenes, fn))(**kw)
    return _cache[name]


def blob(name: str) -> bytes:
    key = ("blob", name)
    if key not in _cache:
        _cache[key] = scene(name).to_bytes()
    return _cache[key]


def qsf_model() -> bytes:
    """The atrium_small atrium (model 0) as a QSF2 file, with the BLAS the oracle builds for it."""
    key = ("qsf",)
    if key not in _cache:
        from oracle_lib import Oracle, qsf_bytes
        blas, root = Oracle(blob("atrium_small")).model_blas(0)
        _cache[key] = qsf_bytes(scene("atrium_small"), 0, blas, root)
    return _cache[key]


# the reference's own QSF2 maps (res/*.qsf), copied beside the reference builds by `make ref`
QSF_MAPS = ["simple", "simpleb"]

# ray queries (sft_raycast_instance): cases and rays per case
RAY_CASES = ["small", "atrium_small", "skinned_small", "variety"]
N_RAYS = 4096


def rays(name: str, n: int = N_RAYS, seed: int = 0):
    """Seeded ray records (oracle_lib.RAY_DTYPE) against the models of a case, with the frame-0
    instance transforms, some scaled by 2 or 0.5: 60% aimed at points of the model's bounds as
    the reference places them (transform rows 0-2, no translation), 20% in random directions,
    10% along coordinate axes (zero direction components), 8% with a short distance limit, and
    two rays of zero direction."""
    from oracle_lib import RAY_DTYPE
    sc = scene(name)
    fr = sc.frames[0]
    insts = [(mi, np.asarray(T, np.float32).reshape(4, 4)) for mi, T, _ in fr.instances]
    bounds = {}
    for mi, _ in insts:
        if mi not in bounds:
            pos = np.concatenate([ms.attr.reshape(ms.n, 10, 64)[:, 0:3].transpose(0, 2, 1).reshape(-1, 3) for ms in sc.models[mi].meshes])
            bounds[mi] = (pos.min(0), pos.max(0))
    rng = np.random.default_rng(seed + sum(name.encode()))
    out = np.zeros(n, RAY_DTYPE)
    cam = np.asarray(fr.cam_pos, np.float32)
    for k in range(n):
        mi, T = insts[rng.integers(len(insts))]
        T = T.copy()
        u = rng.random()
        if u < 0.15:
            T[:3, :3] *= np.float32(2.0)
        elif u < 0.3:
            T[:3, :3] *= np.float32(0.5)
        lo, hi = bounds[mi]
        o = (cam + rng.normal(0, 1.5, 3)).astype(np.float32)
        kind = rng.random()
        if kind < 0.6:
            p = (lo + rng.random(3) * (hi - lo)).astype(np.float32)
            d = (p @ T[:3, :3] - o).astype(np.float32)
        elif kind < 0.8:
            d = rng.normal(0, 1, 3).astype(np.float32)
        else:
            d = np.zeros(3, np.float32)
            d[rng.integers(3)] = np.float32(rng.choice([-1.0, 1.0]) * rng.uniform(0.5, 2.0))
        out[k]["T"] = T.reshape(-1)
        out[k]["o"] = o
        out[k]["d"] = d
        out[k]["max_dist"] = np.float32(rng.uniform(0.5, 3.0) if rng.random() < 0.08 else 1000.0)
        out[k]["model"] = mi
    for k in (n - 2, n - 1):
        out[k]["d"] = 0.0
    return out


# BLAS builds (sft__blas_build_model, sofren2.c:3526-3617) checked model by model: every case's
# models and the edge models of blas_edge_scene
BLAS_CASES = list(CASES) + ["blas_edges"]


def blas_edge_scene():
    """Models at the edges of the BLAS builder (sofren2.c:2895-3062): 5 triangles (one leaf),
    9 (one split), one triangle repeated 3000 times (every centroid equal), 6000 triangles on a
    lattice in the plane z = 1 (no z extent, equal coordinates along x and y), three meshes of
    5, 130 and 7 triangles (padding inside the model's meshlet run), 60000 triangles with
    coordinates on a 1/64 grid (ranges longer than one shared-memory sort, with ties), a single
    triangle, and 40 triangles that are all padding (three equal indices: no BLAS at all)."""
    key = ("blas_edges",)
    if key in _cache:
        return _cache[key]
    sc = scenes.Scene()
    mat = sc.add_material(sc.add_texture(np.full((4, 4), 0xFFFFFFFF, np.uint32)))
    rng = np.random.default_rng(2967)

    def raw(pos, tris):
        pos = np.asarray(pos, np.float32).reshape(-1, 3)
        nrm = np.tile(np.float32([0, 0, 1]), (len(pos), 1))
        return scenes.RawMesh(pos, nrm, np.zeros((len(pos), 2), np.float32), tris)

    def soup(n, grid=None):
        p = rng.uniform(-4, 4, (n, 3)).astype(np.float32)
        e = rng.uniform(-0.3, 0.3, (n, 2, 3)).astype(np.float32)
        v = np.concatenate([p[:, None], p[:, None] + e], axis=1).reshape(-1, 3)
        if grid:
            v = (np.round(v * grid) / grid).astype(np.float32)
        return raw(v, np.arange(3 * n).reshape(-1, 3))

    def add(meshes):
        with np.errstate(invalid="ignore"):   # a lone triangle's cone: sqrt of a rounding-negative 1 - d^2
            ms = [scenes.build_meshlets(m) for m in meshes]
        sc.add_model(scenes.Model(ms, [mat] * len(ms)))

    add([soup(5)])
    add([soup(9)])
    add([raw([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.zeros((3000, 3), np.int64) + np.arange(3))])
    g = np.stack(np.meshgrid(np.arange(41), np.arange(41), indexing="ij"), -1).reshape(-1, 2).astype(np.float32) * 0.25
    lat = np.concatenate([g, np.ones((len(g), 1), np.float32)], 1)
    q = np.array([[i * 41 + j, (i + 1) * 41 + j, i * 41 + j + 1] for i in range(40) for j in range(40)]
                 + [[(i + 1) * 41 + j + 1, i * 41 + j + 1, (i + 1) * 41 + j] for i in range(40) for j in range(40)])
    add([raw(lat, np.concatenate([q, q[: 6000 - len(q)]]) if len(q) < 6000 else q[:6000])])
    add([soup(5), soup(130), soup(7)])
    add([soup(60000, grid=64)])
    add([soup(1)])
    add([raw(rng.uniform(-1, 1, (40, 3)), np.repeat(np.arange(40), 3).reshape(-1, 3))])
    sc.frames.append(scenes._camera_frame(64, 64))
    _cache[key] = sc
    return sc


def blas_blob(name: str) -> bytes:
    if name == "blas_edges":
        key = ("blob", name)
        if key not in _cache:
            _cache[key] = blas_edge_scene().to_bytes()
        return _cache[key]
    return blob(name)


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def n_lights(name: str) -> int:
    return min(64, len(scene(name).frames[0].point_lights))


def digests(frame: dict, live_meshlets: list[int] | None = None, clip_used: int | None = None,
            lights: int = 64) -> dict:
    """Digest of every parity section of a render dump.  ss_cache is digested over the live
    (drawn) meshlets only: culled slots are never written.  The clip pool over its used prefix,
    light visibility over the frame's lights (the reference writes no other column)."""
    out = {k: sha(frame[k]) for k in ("color", "tile_counts", "tile_payloads", "vid")}
    out["light_vis"] = sha(frame["light_vis"].reshape(-1, 64)[:, :lights])
    out["depth"] = sha(frame["depth"].view(np.uint32))
    ss = frame["ss_cache"].view(np.uint32).reshape(-1, 576)
    if live_meshlets is None:
        live_meshlets = np.nonzero(~np.all(ss == 0xFFFFFFFF, axis=1))[0].tolist()
    out["ss_cache_live"] = sha(ss[np.asarray(live_meshlets, dtype=np.int64)]) if len(live_meshlets) else sha(np.zeros(0))
    clip = frame["clip"].view(np.uint32).reshape(-1, 41)
    if clip_used is None:
        clip_used = int(np.count_nonzero(clip[:, 6] != 0))   # inv_w of a used slot is never 0
    out["clip_used"] = clip_used
    out["clip"] = sha(clip[:clip_used])
    return out, live_meshlets
