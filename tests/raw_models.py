"""Raw triangle models for the load-time builders (meshlets, BLAS, shadow proxies), in the input
format of oracle/build_harness.c and tests/model_build.c, and readers of their output.  Shapes
come from the scene generators (sofren2_gb300/scenes.py); seeds fix Welzl's rand() draws."""
from __future__ import annotations

import struct

import numpy as np

from sofren2_gb300 import scenes

F32 = np.float32


def _grid(n: int, half: float, y: float) -> scenes.RawMesh:
    xs = (np.arange(n + 1, dtype=F32) / F32(n) * F32(2 * half) - F32(half)).astype(F32)
    pos = np.array([[xs[i], F32(y), xs[j]] for j in range(n + 1) for i in range(n + 1)], dtype=F32)
    nrm = np.tile(np.array([0.0, 1.0, 0.0], dtype=F32), (len(pos), 1))
    uv = np.array([[F32(i) / F32(8), F32(j) / F32(8)] for j in range(n + 1) for i in range(n + 1)], dtype=F32)
    tris = []
    for j in range(n):
        for i in range(n):
            a, b, c, d = j * (n + 1) + i, j * (n + 1) + i + 1, (j + 1) * (n + 1) + i + 1, (j + 1) * (n + 1) + i
            tris += [[a, b, c], [a, c, d]]
    return scenes.RawMesh(pos, nrm, uv, scenes._orient(pos, nrm, np.array(tris)))


def _soup(n: int, seed: int) -> scenes.RawMesh:
    """Unconnected triangles of random size and direction (no adjacency: every meshlet grows
    from seeds), some of them degenerate (repeated or collinear corners)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-4, 4, size=(n, 1, 3)).astype(F32)
    d = rng.normal(size=(n, 3, 3)).astype(F32) * rng.uniform(0.05, 0.6, size=(n, 1, 1)).astype(F32)
    pos = (c + d).astype(F32).reshape(-1, 3)
    pos[3 * 5 + 1] = pos[3 * 5]                                  # repeated corner
    pos[3 * 9 + 2] = (pos[3 * 9] + pos[3 * 9 + 1]) * F32(0.5)    # collinear
    nrm = rng.normal(size=pos.shape).astype(F32)
    uv = rng.uniform(0, 1, size=(len(pos), 2)).astype(F32)
    return scenes.RawMesh(pos, nrm, uv, np.arange(3 * n).reshape(-1, 3))


def _shared_corners(seed: int) -> scenes.RawMesh:
    """A fan and a strip whose triangles repeat a vertex index within one triangle."""
    m = scenes.uv_sphere(12, 6, 0.7)
    tris = m.tris.copy()
    tris[3, 1] = tris[3, 0]
    tris[17, 2] = tris[17, 1] = tris[17, 0]
    return scenes.RawMesh(m.pos, m.nrm, m.uv, tris)


def models() -> dict:
    """name -> (seed, proxy budget, bones [(parent, bind xyz)], meshes [RawMesh])"""
    hum = [(p, tuple(bp)) for _, p, bp in scenes.HUMANOID_JOINTS]
    boxes = scenes.merge([scenes.box((-1, 0, -1), (1, 0.5, 1)), scenes.box((-0.3, 0.5, -0.3), (0.3, 2.0, 0.3)),
                          scenes.box((2, 0, 2), (2.5, 3, 2.5))])
    return {
        "sphere": (101, 4, [], [scenes.uv_sphere(32, 16, 0.5)]),
        "shapes": (102, 4, [], [scenes.uv_sphere(24, 12, 1.0), boxes, scenes.uv_sphere(8, 4, 0.25)]),
        "ground": (103, 4, [], [_grid(32, 16.0, 0.0)]),
        "humanoid": (104, 10, hum, [scenes.humanoid_mesh(2001)]),
        "humanoid_b3": (105, 3, hum, [scenes.humanoid_mesh(2002)]),
        "soup": (106, 6, [], [_soup(900, 7)]),
        "odd": (107, 2, [], [_shared_corners(3)]),
    }


def blob(name: str) -> bytes:
    seed, budget, bones, meshes = models()[name]
    out = [b"SFTR", struct.pack("<IIiI", 1, seed, budget, len(bones))]
    for parent, bp in bones:
        out.append(struct.pack("<i", parent) + np.asarray(bp, dtype="<f4").tobytes())
    out.append(struct.pack("<I", len(meshes)))
    for m in meshes:
        sk = m.joints is not None
        out.append(struct.pack("<III", len(m.pos), len(m.tris), 1 if sk else 0))
        out += [m.pos.astype("<f4").tobytes(), m.nrm.astype("<f4").tobytes(), m.uv.astype("<f4").tobytes()]
        if sk:
            out += [m.joints.astype("<u2").tobytes(), m.weights.astype("u1").tobytes()]
        out.append(np.asarray(m.tris, dtype="<i4").tobytes())
    return b"".join(out)


def read_output(path: str, name: str, with_blas: bool) -> dict:
    """Meshlets per mesh (Meshlets-like dicts), proxies [n, 8] as u32 words, and (reference
    output only) the BLAS node images and root."""
    raw = open(path, "rb").read()
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a

    meshes = []
    for m in models()[name][3]:
        n = int(take("<u4", 1)[0])
        d = {"n": n, "attr": take("<f4", n * 640).reshape(n, 10, 64), "inds": take("u1", n * 512).reshape(n, 512),
             "cull": take("<f4", n * 8).reshape(n, 8)}
        if m.joints is not None:
            d["joints"] = take("<u2", n * 256).reshape(n, 4, 64)
            d["weights"] = take("u1", n * 256).reshape(n, 4, 64)
            d["bone"] = take("<i4", n)
        meshes.append(d)
    npx = int(take("<u4", 1)[0])
    proxies = take("<u4", npx * 8).reshape(npx, 8)
    out = {"meshes": meshes, "proxies": proxies}
    if with_blas:
        bc, root = (int(x) for x in take("<u4", 2))
        out["blas"] = take("u1", bc * 256).tobytes()
        out["blas_root"] = root
    return out


def meshlet_bytes(out: dict) -> bytes:
    parts = []
    for d in out["meshes"]:
        parts += [np.uint32(d["n"]).tobytes(), d["attr"].tobytes(), d["inds"].tobytes(), d["cull"].tobytes()]
        if "joints" in d:
            parts += [d["joints"].tobytes(), d["weights"].tobytes(), d["bone"].tobytes()]
    return b"".join(parts)


def as_scene_model(out: dict, name: str) -> scenes.Model:
    """The built meshlets as a scene model (for the oracle's BLAS builder or a render)."""
    bones = models()[name][2]
    ms = []
    for d, m in zip(out["meshes"], models()[name][3]):
        skinned = m.joints is not None
        x = scenes.Meshlets(d["n"], skinned)
        x.attr[:] = d["attr"]
        x.inds[:] = d["inds"]
        x.cull[:] = d["cull"]
        if skinned:
            x.joints[:] = d["joints"]
            x.weights[:] = d["weights"]
            x.bone[:] = d["bone"]
        ms.append(x)
    return scenes.Model(ms, [-1] * len(ms), bone_count=len(bones))
