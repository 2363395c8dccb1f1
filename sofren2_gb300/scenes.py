"""Seeded synthetic scenes for the sofren2 render path, serialised as SFTS blobs.

Every number a scene contains is produced with float32 add/sub/mul/div/sqrt and
integer arithmetic only (no libm, no fused multiply-add), so that the same seed
gives the same bits on x86-64 and on aarch64.  Trigonometry and logarithms use
the polynomial approximations below, not numpy's vectorised libm.

The blob layout (little-endian) is read by the C host library
(``csrc/sft_scene.c``), by the CPU oracle and by the reference harness:

    u32 magic 'SFTS', u32 version
    u32 n_textures  { u32 w, h; u32 argb[w*h] }
    u32 n_materials { i32 texture (-1 none); u32 base_color; f32 shininess }
    u32 n_models    { u32 n_meshes, bone_count, n_lightmaps; i32 lightmap_tex[n_lightmaps];
                      u32 n_proxies { f32 posa[3], posb[3], radius; u32 bone }
                      per mesh { u32 meshlet_count; i32 material; u32 lightmap_page; u32 has_skin;
                                 per meshlet: f32 x,y,z,nx,ny,nz,u,v,lu,lv [64 each];
                                              (skin) u16 j0..j3 [64 each]; u8 w0..w3 [64 each];
                                              u8 inds[512]; f32 center[3], radius, axis[3], cutoff;
                                              i32 culling_bone } }
    u32 n_frames    { u32 width, height; f32 cam_pos[3], view[16], proj[16];
                      f32 ambient[3], lightmap_brightness; u32 clear, clear_color, shadows;
                      u32 n_dir  { f32 dir[3], r, g, b, intensity }
                      u32 n_point { f32 pos[3], r, g, b, intensity, radius }
                      u32 n_inst { u32 model; f32 transform[16]; u32 n_bones; f32 bones[16*n] } }

Meshlet conventions follow sofren2 (sofren2.c:914-953): 64 vertices in SoA form,
128 triangles swizzled as 16 batches of [v0 x8, v1 x8, v2 x8, pad x8]; a lane
whose three indices are all zero is padding.  Front faces satisfy
cross(v1 - v0, v2 - v0) . outward_normal > 0 (row-vector transforms, +Z forward,
screen y flipped), which is the orientation the reference's area test keeps.
"""
from __future__ import annotations

import struct
import numpy as np

F32 = np.float32
U32 = np.uint32

MAGIC = 0x53544653
VERSION = 1


# --------------------------------------------------------------------------- PRNG
class Pcg32:
    """PCG-XSH-RR 32-bit generator (O'Neill), seeded through splitmix64."""

    MUL = 6364136223846793005
    MASK = (1 << 64) - 1

    def __init__(self, seed: int, stream: int = 0):
        s = (seed * 0x9E3779B97F4A7C15 + 0xBF58476D1CE4E5B9) & self.MASK
        s ^= s >> 31
        self.inc = ((stream << 1) | 1) & self.MASK
        self.state = 0
        self.next_u32()
        self.state = (self.state + s) & self.MASK
        self.next_u32()

    def next_u32(self) -> int:
        old = self.state
        self.state = (old * self.MUL + self.inc) & self.MASK
        xorshifted = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xorshifted >> rot) | (xorshifted << ((-rot) & 31))) & 0xFFFFFFFF

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> np.float32:
        """float32 in [lo, hi): 24 random bits scaled exactly, then one mul+add."""
        u = F32(self.next_u32() >> 8) * F32(1.0 / 16777216.0)
        return F32(F32(lo) + F32(F32(F32(hi) - F32(lo)) * u))

    def u32_array(self, n: int) -> np.ndarray:
        return np.array([self.next_u32() for _ in range(n)], dtype=np.uint32)


# ------------------------------------------------------------- deterministic math
_PI = F32(3.14159265358979)
_TWO_PI = F32(6.28318530717959)
_HALF_PI = F32(1.57079632679490)


def _poly(x, coeffs):
    acc = np.full_like(x, F32(coeffs[0]))
    for c in coeffs[1:]:
        acc = (acc * x + F32(c)).astype(F32)
    return acc


def dsin(a) -> np.ndarray:
    """sin for float32 arrays: reduction to [-pi/2, pi/2] then an odd Taylor polynomial."""
    x = np.asarray(a, dtype=F32)
    k = np.floor((x / _TWO_PI + F32(0.5)).astype(F32)).astype(F32)
    r = (x - (k * _TWO_PI).astype(F32)).astype(F32)            # [-pi, pi)
    r = np.where(r > _HALF_PI, (_PI - r).astype(F32), r).astype(F32)
    r = np.where(r < -_HALF_PI, (-_PI - r).astype(F32), r).astype(F32)
    r2 = (r * r).astype(F32)
    p = _poly(r2, [-1.0 / 39916800.0, 1.0 / 362880.0, -1.0 / 5040.0, 1.0 / 120.0, -1.0 / 6.0, 1.0])
    return (r * p).astype(F32)


def dcos(a) -> np.ndarray:
    return dsin((np.asarray(a, dtype=F32) + _HALF_PI).astype(F32))


def dlog(a) -> np.ndarray:
    """natural log for positive float32 arrays via exponent split and atanh series."""
    x = np.asarray(a, dtype=F32)
    bits = x.view(np.uint32).astype(np.int64)
    e = ((bits >> 23) & 0xFF) - 127
    m = ((bits & 0x7FFFFF) | (127 << 23)).astype(np.uint32).view(F32)   # [1, 2)
    big = m > F32(1.41421356)
    m = np.where(big, (m * F32(0.5)).astype(F32), m).astype(F32)
    e = np.where(big, e + 1, e)
    t = ((m - F32(1.0)) / (m + F32(1.0))).astype(F32)
    t2 = (t * t).astype(F32)
    s = _poly(t2, [1.0 / 11.0, 1.0 / 9.0, 1.0 / 7.0, 1.0 / 5.0, 1.0 / 3.0, 1.0])
    ln_m = (F32(2.0) * (t * s).astype(F32)).astype(F32)
    return (ln_m + (e.astype(F32) * F32(0.693147180559945)).astype(F32)).astype(F32)


def f32(x) -> np.float32:
    return F32(x)


# --------------------------------------------------------------------- matrices
def mat_identity() -> np.ndarray:
    return np.eye(4, dtype=F32)


def mat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Row-major product with the same left-to-right sums as sofren2's sft_m_mul (sofren2.c:1668)."""
    r = np.zeros((4, 4), dtype=F32)
    for i in range(4):
        for j in range(4):
            acc = F32(a[i, 0] * b[0, j])
            for k in range(1, 4):
                acc = F32(acc + F32(a[i, k] * b[k, j]))
            r[i, j] = acc
    return r


def mat_translate(x, y, z) -> np.ndarray:
    m = mat_identity()
    m[3, 0], m[3, 1], m[3, 2] = F32(x), F32(y), F32(z)
    return m


def mat_scale(s) -> np.ndarray:
    m = mat_identity()
    m[0, 0] = m[1, 1] = m[2, 2] = F32(s)
    return m


def mat_rot_y(a) -> np.ndarray:
    c, s = dcos(F32(a)), dsin(F32(a))
    m = mat_identity()
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    return m


def mat_rot_x(a) -> np.ndarray:
    c, s = dcos(F32(a)), dsin(F32(a))
    m = mat_identity()
    m[1, 1], m[1, 2], m[2, 1], m[2, 2] = c, s, -s, c
    return m


def mat_rot_z(a) -> np.ndarray:
    c, s = dcos(F32(a)), dsin(F32(a))
    m = mat_identity()
    m[0, 0], m[0, 1], m[1, 0], m[1, 1] = c, s, -s, c
    return m


def _dot3(a, b) -> np.float32:
    return F32(F32(F32(a[0] * b[0]) + F32(a[1] * b[1])) + F32(a[2] * b[2]))


def _norm3(v: np.ndarray) -> np.ndarray:
    v = np.asarray(v, dtype=F32)
    l = np.sqrt((v[0] * v[0] + v[1] * v[1] + v[2] * v[2]).astype(F32)).astype(F32)
    return (v / l).astype(F32)


def _cross3(a, b) -> np.ndarray:
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], dtype=F32)


def view_look_at(pos, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Camera matrix laid out like sofren2's sft_m_view_look_at (sofren2.c:1737)."""
    pos = np.asarray(pos, dtype=F32)
    fwd = _norm3(np.asarray(target, dtype=F32) - pos)
    up = np.asarray(up, dtype=F32)
    up = _norm3(up - fwd * _dot3(up, fwd))
    right = _cross3(up, fwd)
    m = mat_identity()
    m[0, 0], m[0, 1], m[0, 2] = right[0], up[0], fwd[0]
    m[1, 0], m[1, 1], m[1, 2] = right[1], up[1], fwd[1]
    m[2, 0], m[2, 1], m[2, 2] = right[2], up[2], fwd[2]
    m[3, 0] = -_dot3(pos, right)
    m[3, 1] = -_dot3(pos, up)
    m[3, 2] = -_dot3(pos, fwd)
    return m


def proj(fov_deg, aspect, near, far) -> np.ndarray:
    """Perspective matrix laid out like sofren2's sft_m_proj (sofren2.c:1646)."""
    half = F32(F32(fov_deg) * F32(0.5) / F32(180.0) * _PI)
    f = F32(dcos(half) / dsin(half))
    m = np.zeros((4, 4), dtype=F32)
    m[0, 0] = F32(f / F32(aspect))
    m[1, 1] = f
    m[2, 2] = F32(F32(far) / F32(F32(far) - F32(near)))
    m[3, 2] = F32(F32(-F32(far) * F32(near)) / F32(F32(far) - F32(near)))
    m[2, 3] = F32(1.0)
    return m


# --------------------------------------------------------------------- textures
def _hash_lattice(ix: np.ndarray, iy: np.ndarray, seed: int, channel: int) -> np.ndarray:
    h = (ix.astype(np.uint64) * np.uint64(0x8DA6B343) + iy.astype(np.uint64) * np.uint64(0xD8163841)
         + np.uint64((seed * 0x27D4EB2D + channel * 0x165667B1) & 0xFFFFFFFF)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    h = (h * np.uint64(0x2C1B3C6D)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(12)
    h = (h * np.uint64(0x297A2D39)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    return (h & np.uint64(0xFF)).astype(F32)


def value_noise_texture(w: int, h: int, seed: int, lattice: int = 16) -> np.ndarray:
    """ARGB8888 value noise: integer lattice every `lattice` px, smoothstep-bilinear per channel."""
    ys, xs = np.mgrid[0:h, 0:w]
    gx, gy = xs // lattice, ys // lattice
    fx = ((xs % lattice).astype(F32) / F32(lattice)).astype(F32)
    fy = ((ys % lattice).astype(F32) / F32(lattice)).astype(F32)
    sx = (fx * fx * (F32(3.0) - F32(2.0) * fx)).astype(F32)
    sy = (fy * fy * (F32(3.0) - F32(2.0) * fy)).astype(F32)
    out = np.full((h, w), 0xFF000000, dtype=np.uint32)
    for ch, shift in ((0, 16), (1, 8), (2, 0)):
        a = _hash_lattice(gx, gy, seed, ch)
        b = _hash_lattice(gx + 1, gy, seed, ch)
        c = _hash_lattice(gx, gy + 1, seed, ch)
        d = _hash_lattice(gx + 1, gy + 1, seed, ch)
        top = (a + (b - a) * sx).astype(F32)
        bot = (c + (d - c) * sx).astype(F32)
        v = (top + (bot - top) * sy).astype(F32)
        out |= (np.clip(v, 0, 255).astype(np.uint32) & 0xFF) << np.uint32(shift)
    return out


# ------------------------------------------------------------------------ meshes
class RawMesh:
    """Indexed triangle mesh with float32 attributes (and optional skin)."""

    def __init__(self, pos, nrm, uv, tris, luv=None, joints=None, weights=None):
        self.pos = np.asarray(pos, dtype=F32).reshape(-1, 3)
        self.nrm = np.asarray(nrm, dtype=F32).reshape(-1, 3)
        self.uv = np.asarray(uv, dtype=F32).reshape(-1, 2)
        self.luv = (np.zeros((len(self.pos), 2), dtype=F32) if luv is None
                    else np.asarray(luv, dtype=F32).reshape(-1, 2))
        self.tris = np.asarray(tris, dtype=np.int64).reshape(-1, 3)
        self.joints = None if joints is None else np.asarray(joints, dtype=np.uint16).reshape(-1, 4)
        self.weights = None if weights is None else np.asarray(weights, dtype=np.uint8).reshape(-1, 4)


def _orient(pos, nrm, tris):
    """Flip triangles whose geometric normal disagrees with the mean vertex normal."""
    p0, p1, p2 = pos[tris[:, 0]], pos[tris[:, 1]], pos[tris[:, 2]]
    gn = np.cross((p1 - p0).astype(F32), (p2 - p0).astype(F32)).astype(F32)
    vn = (nrm[tris[:, 0]] + nrm[tris[:, 1]] + nrm[tris[:, 2]]).astype(F32)
    flip = (gn[:, 0] * vn[:, 0] + gn[:, 1] * vn[:, 1] + gn[:, 2] * vn[:, 2]) < 0
    t = tris.copy()
    t[flip, 1], t[flip, 2] = tris[flip, 2], tris[flip, 1]
    return t


def uv_sphere(slices: int = 32, bands: int = 16, radius: float = 0.5) -> RawMesh:
    pos, nrm, uv = [], [], []
    for b in range(bands + 1):
        th = F32(F32(b) / F32(bands) * _PI)
        st, ct = dsin(th), dcos(th)
        for s in range(slices + 1):
            ph = F32(F32(s) / F32(slices) * _TWO_PI)
            sp, cp = dsin(ph), dcos(ph)
            n = np.array([st * cp, ct, st * sp], dtype=F32)
            nrm.append(n)
            pos.append((n * F32(radius)).astype(F32))
            uv.append([F32(s) / F32(slices), F32(b) / F32(bands)])
    tris = []
    w = slices + 1
    for b in range(bands):
        for s in range(slices):
            a, c = b * w + s, (b + 1) * w + s
            if b != 0:
                tris.append([a, a + 1, c + 1])
            if b != bands - 1:
                tris.append([a, c + 1, c])
    pos, nrm = np.array(pos, dtype=F32), np.array(nrm, dtype=F32)
    tris = _orient(pos, nrm, np.array(tris))
    return RawMesh(pos, nrm, np.array(uv, dtype=F32), tris)


def box(lo, hi, uv_scale: float = 1.0) -> RawMesh:
    """Axis-aligned box with 4 vertices per face (flat normals)."""
    lo, hi = np.asarray(lo, dtype=F32), np.asarray(hi, dtype=F32)
    faces = [((0, -1), (2, 1)), ((0, 1), (2, 1)), ((1, -1), (0, 2)), ((1, 1), (0, 2)), ((2, -1), (0, 1)), ((2, 1), (0, 1))]
    pos, nrm, uv, tris = [], [], [], []
    for (ax, sgn), (ua, va) in faces:
        base = len(pos)
        n = np.zeros(3, dtype=F32)
        n[ax] = F32(sgn)
        for (cu, cv) in ((0, 0), (0, 1), (1, 1), (1, 0)):
            p = np.zeros(3, dtype=F32)
            p[ax] = hi[ax] if sgn > 0 else lo[ax]
            p[ua] = hi[ua] if cu else lo[ua]
            p[va] = hi[va] if cv else lo[va]
            pos.append(p)
            nrm.append(n)
            uv.append([F32(cu) * F32(uv_scale), F32(cv) * F32(uv_scale)])
        tris += [[base, base + 1, base + 2], [base, base + 2, base + 3]]
    pos, nrm = np.array(pos, dtype=F32), np.array(nrm, dtype=F32)
    return RawMesh(pos, nrm, np.array(uv, dtype=F32), _orient(pos, nrm, np.array(tris)))


def merge(meshes) -> RawMesh:
    pos, nrm, uv, luv, tris, j, w = [], [], [], [], [], [], []
    off = 0
    skinned = any(m.joints is not None for m in meshes)
    for m in meshes:
        pos.append(m.pos); nrm.append(m.nrm); uv.append(m.uv); luv.append(m.luv)
        tris.append(m.tris + off)
        if skinned:
            j.append(m.joints if m.joints is not None else np.zeros((len(m.pos), 4), np.uint16))
            w.append(m.weights if m.weights is not None else np.tile(np.array([255, 0, 0, 0], np.uint8), (len(m.pos), 1)))
        off += len(m.pos)
    return RawMesh(np.concatenate(pos), np.concatenate(nrm), np.concatenate(uv), np.concatenate(tris),
                   np.concatenate(luv), np.concatenate(j) if skinned else None, np.concatenate(w) if skinned else None)


# ---------------------------------------------------------------------- meshlets
class Meshlets:
    """Meshlet arrays for one mesh in the layout sofren2 consumes (sofren2.c:914-953, 1071-1092)."""

    def __init__(self, n: int, skinned: bool):
        self.n = n
        self.attr = np.zeros((n, 10, 64), dtype=F32)      # x y z nx ny nz u v lu lv
        self.joints = np.zeros((n, 4, 64), dtype=np.uint16) if skinned else None
        self.weights = np.zeros((n, 4, 64), dtype=np.uint8) if skinned else None
        self.inds = np.zeros((n, 512), dtype=np.uint8)
        self.cull = np.zeros((n, 8), dtype=F32)           # center xyz, radius, axis xyz, cutoff
        self.bone = np.full(n, -1, dtype=np.int32)
        self.tri_count = np.zeros(n, dtype=np.int32)


def build_meshlets(mesh: RawMesh, max_verts: int = 64, max_tris: int = 128) -> Meshlets:
    """Greedy in-order packing: a meshlet closes when the next triangle would exceed 64 verts or 128 tris."""
    groups = []
    cur_tris, cur_map = [], {}
    for t in mesh.tris:
        new = [v for v in dict.fromkeys(t.tolist()) if v not in cur_map]
        if len(cur_tris) + 1 > max_tris or len(cur_map) + len(new) > max_verts:
            groups.append((cur_tris, cur_map))
            cur_tris, cur_map = [], {}
            new = list(dict.fromkeys(t.tolist()))
        for v in new:
            cur_map[v] = len(cur_map)
        cur_tris.append([cur_map[v] for v in t.tolist()])
    if cur_tris:
        groups.append((cur_tris, cur_map))

    skinned = mesh.joints is not None
    out = Meshlets(len(groups), skinned)
    for mi, (tris, vmap) in enumerate(groups):
        verts = np.array(list(vmap.keys()), dtype=np.int64)
        nv = len(verts)
        out.attr[mi, 0:3, :nv] = mesh.pos[verts].T
        out.attr[mi, 3:6, :nv] = mesh.nrm[verts].T
        out.attr[mi, 6:8, :nv] = mesh.uv[verts].T
        out.attr[mi, 8:10, :nv] = mesh.luv[verts].T
        if skinned:
            out.joints[mi, :, :nv] = mesh.joints[verts].T
            out.weights[mi, :, :nv] = mesh.weights[verts].T
            wsum = np.zeros(int(mesh.joints.max()) + 1, dtype=np.int64)
            for k in range(4):
                np.add.at(wsum, mesh.joints[verts, k].astype(np.int64), mesh.weights[verts, k].astype(np.int64))
            out.bone[mi] = int(np.argmax(wsum))
        tri = np.array(tris, dtype=np.int64)
        out.tri_count[mi] = len(tri)
        for ti, (a, b, c) in enumerate(tri):
            batch, lane = divmod(ti, 8)
            out.inds[mi, batch * 32 + lane] = a
            out.inds[mi, batch * 32 + 8 + lane] = b
            out.inds[mi, batch * 32 + 16 + lane] = c
        p = mesh.pos[verts]
        lo, hi = p.min(axis=0), p.max(axis=0)
        ctr = ((lo + hi) * F32(0.5)).astype(F32)
        d = (p - ctr).astype(F32)
        rad = F32(np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]).astype(F32)).max())
        rad = F32(rad * F32(1.0001) + F32(1e-5))
        gp = mesh.pos
        t3 = np.array([[verts[a], verts[b], verts[c]] for a, b, c in tri])
        fn = np.cross((gp[t3[:, 1]] - gp[t3[:, 0]]).astype(F32), (gp[t3[:, 2]] - gp[t3[:, 0]]).astype(F32)).astype(F32)
        fl = np.sqrt((fn[:, 0] * fn[:, 0] + fn[:, 1] * fn[:, 1] + fn[:, 2] * fn[:, 2]).astype(F32)).astype(F32)
        fn = (fn / np.maximum(fl, F32(1e-20))[:, None]).astype(F32)
        axis = np.zeros(3, dtype=F32)
        for row in fn:
            axis = (axis + row).astype(F32)
        al = F32(np.sqrt(_dot3(axis, axis)))
        if al > F32(1e-6) and not skinned:
            axis = (axis / al).astype(F32)
            mindp = F32((fn[:, 0] * axis[0] + fn[:, 1] * axis[1] + fn[:, 2] * axis[2]).astype(F32).min())
            cutoff = F32(np.sqrt(F32(F32(1.0) - mindp * mindp))) if mindp > F32(0.1) else F32(2.0)
        else:
            axis = np.array([0, 0, 1], dtype=F32)
            cutoff = F32(2.0)
        out.cull[mi] = [ctr[0], ctr[1], ctr[2], rad, axis[0], axis[1], axis[2], cutoff]
    return out


# ------------------------------------------------------------------------ scene
class Model:
    def __init__(self, meshes, materials, bone_count=0, proxies=(), lightmaps=(), lightmap_pages=None):
        self.meshes = meshes                  # list[Meshlets]
        self.materials = materials            # material index per mesh
        self.bone_count = bone_count
        self.proxies = list(proxies)          # (posa, posb, radius, bone)
        self.lightmaps = list(lightmaps)      # texture indices
        self.lightmap_pages = lightmap_pages or [0xFFFFFFFF] * len(meshes)


class Frame:
    def __init__(self, width, height, cam_pos, view, projm):
        self.width, self.height = width, height
        self.cam_pos = np.asarray(cam_pos, dtype=F32)
        self.view, self.proj = view, projm
        self.ambient = np.array([0.1, 0.1, 0.1], dtype=F32)
        self.lightmap_brightness = F32(1.5)
        self.clear, self.clear_color, self.shadows = 1, 0xFF222222, 1
        self.dir_lights = []                  # (dir3, r, g, b, intensity)
        self.point_lights = []                # (pos3, r, g, b, intensity, radius)
        self.instances = []                   # (model, transform4x4, bones[n,4,4] or None)


class Scene:
    def __init__(self):
        self.textures, self.materials, self.models, self.frames = [], [], [], []

    def add_texture(self, argb: np.ndarray) -> int:
        self.textures.append(np.ascontiguousarray(argb, dtype=np.uint32))
        return len(self.textures) - 1

    def add_material(self, tex: int, base_color: int = 0xFFFFFFFF, shininess: float = 16.0) -> int:
        self.materials.append((tex, base_color, F32(shininess)))
        return len(self.materials) - 1

    def add_model(self, model: Model) -> int:
        self.models.append(model)
        return len(self.models) - 1

    def to_bytes(self) -> bytes:
        out = [struct.pack("<II", MAGIC, VERSION), struct.pack("<I", len(self.textures))]
        for t in self.textures:
            out.append(struct.pack("<II", t.shape[1], t.shape[0]))
            out.append(t.astype("<u4").tobytes())
        out.append(struct.pack("<I", len(self.materials)))
        for tex, base, shin in self.materials:
            out.append(struct.pack("<iIf", tex, base, shin))
        out.append(struct.pack("<I", len(self.models)))
        for m in self.models:
            out.append(struct.pack("<III", len(m.meshes), m.bone_count, len(m.lightmaps)))
            out.append(np.asarray(m.lightmaps, dtype="<i4").tobytes())
            out.append(struct.pack("<I", len(m.proxies)))
            for pa, pb, r, bone in m.proxies:
                out.append(np.asarray([*pa, *pb, r], dtype="<f4").tobytes() + struct.pack("<I", bone & 0xFFFFFFFF))
            for ms, mat, page in zip(m.meshes, m.materials, m.lightmap_pages):
                skin = ms.joints is not None
                out.append(struct.pack("<IiII", ms.n, mat, page, 1 if skin else 0))
                for i in range(ms.n):
                    out.append(ms.attr[i].astype("<f4").tobytes())
                    if skin:
                        out.append(ms.joints[i].astype("<u2").tobytes())
                        out.append(ms.weights[i].astype("u1").tobytes())
                    out.append(ms.inds[i].tobytes())
                    out.append(ms.cull[i].astype("<f4").tobytes())
                    out.append(struct.pack("<i", int(ms.bone[i])))
        out.append(struct.pack("<I", len(self.frames)))
        for f in self.frames:
            out.append(struct.pack("<II", f.width, f.height))
            out.append(f.cam_pos.astype("<f4").tobytes() + f.view.astype("<f4").tobytes() + f.proj.astype("<f4").tobytes())
            out.append(f.ambient.astype("<f4").tobytes() + struct.pack("<f", f.lightmap_brightness))
            out.append(struct.pack("<III", f.clear, f.clear_color, f.shadows))
            out.append(struct.pack("<I", len(f.dir_lights)))
            for d, r, g, b, it in f.dir_lights:
                out.append(np.asarray([*d, r, g, b, it], dtype="<f4").tobytes())
            out.append(struct.pack("<I", len(f.point_lights)))
            for p, r, g, b, it, rad in f.point_lights:
                out.append(np.asarray([*p, r, g, b, it, rad], dtype="<f4").tobytes())
            out.append(struct.pack("<I", len(f.instances)))
            for mi, tr, bones in f.instances:
                nb = 0 if bones is None else len(bones)
                out.append(struct.pack("<I", mi) + np.asarray(tr, dtype="<f4").tobytes() + struct.pack("<I", nb))
                if nb:
                    out.append(np.asarray(bones, dtype="<f4").tobytes())
        return b"".join(out)


# ------------------------------------------------------------------- configs
def _camera_frame(width, height, cam_pos=(0.0, 0.0, 0.0), target=(0.0, 0.0, 1.0), fov=60.0, near=0.1, far=100.0):
    f = Frame(width, height, cam_pos, view_look_at(cam_pos, target), None)
    f.proj = proj(fov, F32(width) / F32(height), near, far)
    return f


def static_shapes_scene(width=640, height=360, seed=1001, n_spheres=16, n_cubes=16, tex_size=256,
                        n_lights=1, cube_center=(0.0, 0.0, 25.0), cube_half=10.0, slices=32, bands=16,
                        frames=1) -> Scene:
    """Spheres and unit cubes with per-instance value-noise textures lit by point lights.

    Placement per instance: position uniform in a cube of half-size `cube_half` about
    `cube_center`, yaw U[0, 2pi), uniform scale U[0.5, 2]; one capsule shadow proxy per
    model fitted to the shape."""
    rng = Pcg32(seed)
    sc = Scene()
    sphere_ml = build_meshlets(uv_sphere(slices, bands, 0.5))
    cube_ml = build_meshlets(box((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)))
    cx, cy, cz = (F32(v) for v in cube_center)
    insts = []
    for i in range(n_spheres + n_cubes):
        is_sphere = i < n_spheres
        tex = sc.add_texture(value_noise_texture(tex_size, tex_size, seed * 131 + i))
        mat = sc.add_material(tex, 0xFFFFFFFF, 16.0)
        if is_sphere:
            proxies = [((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.5, 0xFFFFFFFF)]
            mdl = Model([sphere_ml], [mat], proxies=proxies)
        else:
            proxies = [((0.0, -0.25, 0.0), (0.0, 0.25, 0.0), 0.45, 0xFFFFFFFF)]
            mdl = Model([cube_ml], [mat], proxies=proxies)
        mi = sc.add_model(mdl)
        px = F32(cx + rng.uniform(-cube_half, cube_half))
        py = F32(cy + rng.uniform(-cube_half, cube_half))
        pz = F32(cz + rng.uniform(-cube_half, cube_half))
        yaw = rng.uniform(0.0, 6.28318530717959)
        s = rng.uniform(0.5, 2.0)
        tr = mat_mul(mat_mul(mat_scale(s), mat_rot_y(yaw)), mat_translate(px, py, pz))
        insts.append((mi, tr, None))
    lights = []
    for _ in range(n_lights):
        # Lights sit well above the object cube: sofren2's packet frustum (sofren2.c:4027-4048)
        # leaves side planes uninitialised when a light lies inside a proxy batch's bounding box.
        lp = (F32(cx + rng.uniform(-0.1 * cube_half, 0.1 * cube_half)), F32(cy + F32(3.0 * cube_half)),
              F32(cz + rng.uniform(-0.1 * cube_half, 0.1 * cube_half)))
        lights.append((lp, F32(1.0), F32(0.95), F32(0.9), F32(1.0), F32(6.0 * cube_half)))
    for fi in range(frames):
        fr = _camera_frame(width, height)
        fr.ambient = np.array([0.2, 0.2, 0.22], dtype=F32)
        fr.point_lights = list(lights)
        fr.instances = list(insts)
        sc.frames.append(fr)
    return sc


def config1(width=640, height=360, seed=1001) -> Scene:
    """Plain static frame: 16 UV-spheres (32x16) + 16 unit cubes, 256x256 textures, one point light,
    camera at the origin looking +Z, 60 degree fov, near 0.1, far 100."""
    return static_shapes_scene(width, height, seed)


# ------------------------------------------------------------------ capsules and skinning
def _frame_for(axis: np.ndarray):
    """Orthonormal (u, v) perpendicular to a unit axis, built from the least-aligned cardinal axis."""
    ax = np.abs(axis)
    card = np.zeros(3, dtype=F32)
    card[int(np.argmin(ax))] = F32(1.0)
    u = _norm3(_cross3(axis, card))
    v = _cross3(axis, u)
    return u, v


def capsule(a, b, radius, slices=16, rings=5, body=4, caps=True) -> RawMesh:
    """Capsule (or open cylinder when caps=False) from a to b; rows of vertices joined by quads,
    pole triangles skipped."""
    a, b = np.asarray(a, dtype=F32), np.asarray(b, dtype=F32)
    d = (b - a).astype(F32)
    axis = _norm3(d)
    u, v = _frame_for(axis)
    rows = []   # (centre, phi)
    if caps:
        for i in range(rings + 1):
            rows.append((a, F32(-_HALF_PI + _HALF_PI * F32(i) / F32(rings))))
    else:
        rows.append((a, F32(0.0)))
    for j in range(1, body):
        t = F32(F32(j) / F32(body))
        rows.append(((a + d * t).astype(F32), F32(0.0)))
    if caps:
        for i in range(rings + 1):
            rows.append((b, F32(_HALF_PI * F32(i) / F32(rings))))
    else:
        rows.append((b, F32(0.0)))
    pos, nrm, uv = [], [], []
    th = (np.arange(slices + 1, dtype=F32) / F32(slices) * _TWO_PI).astype(F32)
    ct, st = dcos(th), dsin(th)
    for ri, (c, phi) in enumerate(rows):
        cp, sp = dcos(phi), dsin(phi)
        ring = ((ct[:, None] * u[None, :] + st[:, None] * v[None, :]).astype(F32) * cp + axis[None, :] * sp).astype(F32)
        nrm.append(ring)
        pos.append((c[None, :] + ring * F32(radius)).astype(F32))
        uv.append(np.stack([th / _TWO_PI, np.full(slices + 1, F32(ri) / F32(len(rows) - 1), dtype=F32)], axis=1))
    pos, nrm, uv = np.concatenate(pos), np.concatenate(nrm), np.concatenate(uv).astype(F32)
    w = slices + 1
    tris = []
    nr = len(rows)
    for r in range(nr - 1):
        pole_lo = caps and r == 0
        pole_hi = caps and r == nr - 2
        for s in range(slices):
            p0, p1, p2, p3 = r * w + s, r * w + s + 1, (r + 1) * w + s + 1, (r + 1) * w + s
            if not pole_lo:
                tris.append([p0, p1, p2])
            if not pole_hi:
                tris.append([p0, p2, p3])
    tris = _orient(pos, nrm, np.array(tris))
    return RawMesh(pos, nrm, uv, tris)


HUMANOID_JOINTS = [   # (name, parent, bind position)
    ("pelvis", -1, (0.0, 1.0, 0.0)), ("spine1", 0, (0.0, 1.15, 0.0)), ("spine2", 1, (0.0, 1.3, 0.0)),
    ("chest", 2, (0.0, 1.45, 0.0)), ("neck", 3, (0.0, 1.58, 0.0)), ("head", 4, (0.0, 1.7, 0.0)),
    ("l_clav", 3, (0.08, 1.5, 0.0)), ("l_upperarm", 6, (0.2, 1.48, 0.0)), ("l_forearm", 7, (0.45, 1.48, 0.0)),
    ("l_hand", 8, (0.68, 1.48, 0.0)), ("r_clav", 3, (-0.08, 1.5, 0.0)), ("r_upperarm", 10, (-0.2, 1.48, 0.0)),
    ("r_forearm", 11, (-0.45, 1.48, 0.0)), ("r_hand", 12, (-0.68, 1.48, 0.0)), ("l_thigh", 0, (0.1, 0.95, 0.0)),
    ("l_shin", 14, (0.1, 0.52, 0.0)), ("l_foot", 15, (0.1, 0.08, 0.0)), ("l_toe", 16, (0.1, 0.03, -0.15)),
    ("r_thigh", 0, (-0.1, 0.95, 0.0)), ("r_shin", 18, (-0.1, 0.52, 0.0)), ("r_foot", 19, (-0.1, 0.08, 0.0)),
    ("r_toe", 20, (-0.1, 0.03, -0.15)),
]

# body parts: (a, b, radius, caps); shadow proxies are the head, torso, arm and leg capsules
HUMANOID_PARTS = [
    ((0.0, 0.95, 0.0), (0.0, 1.5, 0.0), 0.16, True), ((0.0, 1.62, 0.0), (0.0, 1.8, 0.0), 0.11, True),
    ((0.0, 1.52, 0.0), (0.0, 1.64, 0.0), 0.05, False),
    ((0.2, 1.48, 0.0), (0.45, 1.48, 0.0), 0.055, True), ((0.45, 1.48, 0.0), (0.68, 1.48, 0.0), 0.045, True),
    ((0.68, 1.48, 0.0), (0.78, 1.48, 0.0), 0.04, True),
    ((-0.2, 1.48, 0.0), (-0.45, 1.48, 0.0), 0.055, True), ((-0.45, 1.48, 0.0), (-0.68, 1.48, 0.0), 0.045, True),
    ((-0.68, 1.48, 0.0), (-0.78, 1.48, 0.0), 0.04, True),
    ((0.1, 0.95, 0.0), (0.1, 0.52, 0.0), 0.08, True), ((0.1, 0.52, 0.0), (0.1, 0.1, 0.0), 0.06, True),
    ((0.1, 0.06, 0.0), (0.1, 0.05, -0.18), 0.045, True),
    ((-0.1, 0.95, 0.0), (-0.1, 0.52, 0.0), 0.08, True), ((-0.1, 0.52, 0.0), (-0.1, 0.1, 0.0), 0.06, True),
    ((-0.1, 0.06, 0.0), (-0.1, 0.05, -0.18), 0.045, True),
]
HUMANOID_PROXIES = [   # (part index, bone)
    (1, 5), (0, 2), (3, 7), (4, 8), (6, 11), (7, 12), (9, 14), (10, 15), (12, 18), (13, 19),
]


def humanoid_mesh(seed: int) -> RawMesh:
    """About 6k triangles of capsules and cylinders, skinned to the 4 nearest of 22 joints with
    Dirichlet(1) weights quantised to u8."""
    parts = [capsule(a, b, r, slices=16, rings=5, body=4, caps=c) for a, b, r, c in HUMANOID_PARTS]
    m = merge(parts)
    rng = Pcg32(seed, 7)
    jp = np.array([p for _, _, p in HUMANOID_JOINTS], dtype=F32)
    n = len(m.pos)
    joints = np.zeros((n, 4), dtype=np.uint16)
    weights = np.zeros((n, 4), dtype=np.uint8)
    for i in range(n):
        d = (m.pos[i][None, :] - jp).astype(F32)
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]).astype(F32)
        near = np.argsort(d2, kind="stable")[:4]
        u = np.array([F32(((rng.next_u32() >> 8) + 1)) * F32(1.0 / 16777216.0) for _ in range(4)], dtype=F32)
        e = (-dlog(u)).astype(F32)
        s = F32(F32(F32(e[0] + e[1]) + e[2]) + e[3])
        w = (e / s).astype(F32)
        joints[i] = near
        weights[i] = np.floor((w * F32(255.0) + F32(0.5)).astype(F32)).astype(np.uint8)
    m.joints, m.weights = joints, weights
    return m


def _quat_axis_angle(axis, ang):
    h = F32(F32(ang) * F32(0.5))
    s, c = dsin(h), dcos(h)
    return np.array([axis[0] * s, axis[1] * s, axis[2] * s, c], dtype=F32)


def _quat_to_mat(q):
    """sft_m_from_quat layout (sofren2.c:1822)."""
    x, y, z, w = (F32(v) for v in q)
    x2, y2, z2 = F32(x + x), F32(y + y), F32(z + z)
    xx, xy, xz = F32(x * x2), F32(x * y2), F32(x * z2)
    yy, yz, zz = F32(y * y2), F32(y * z2), F32(z * z2)
    wx, wy, wz = F32(w * x2), F32(w * y2), F32(w * z2)
    m = mat_identity()
    m[0, 0], m[0, 1], m[0, 2] = F32(1.0) - F32(yy + zz), F32(xy + wz), F32(xz - wy)
    m[1, 0], m[1, 1], m[1, 2] = F32(xy - wz), F32(1.0) - F32(xx + zz), F32(yz + wx)
    m[2, 0], m[2, 1], m[2, 2] = F32(xz + wy), F32(yz - wx), F32(1.0) - F32(xx + yy)
    return m


class HumanoidAnim:
    """30 keyframes per joint of a sinusoidal local rotation (amplitude U[0, 0.6] rad, seeded
    axis and phase), normalised-linear interpolation between keys."""

    def __init__(self, seed: int, keys: int = 30):
        rng = Pcg32(seed, 11)
        self.keys = keys
        self.q = np.zeros((len(HUMANOID_JOINTS), keys, 4), dtype=F32)
        for j in range(len(HUMANOID_JOINTS)):
            ax = _norm3(np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-1, 1)], dtype=F32) + F32(1e-3))
            amp, ph = rng.uniform(0.0, 0.6), rng.uniform(0.0, 1.0)
            for k in range(keys):
                t = F32(F32(k) / F32(keys - 1))
                ang = F32(amp * dsin(F32(_TWO_PI * F32(t + ph))))
                self.q[j, k] = _quat_axis_angle(ax, ang)

    def pose(self, t: float) -> np.ndarray:
        """Posed bone matrices (inverse bind x global), [22, 4, 4] float32, at clip time t in [0, 1)."""
        ft = F32(F32(t) * F32(self.keys - 1))
        k0 = int(np.floor(ft)) % (self.keys - 1)
        a = F32(ft - F32(k0))
        glob = []
        out = np.zeros((len(HUMANOID_JOINTS), 4, 4), dtype=F32)
        for j, (_, parent, bp) in enumerate(HUMANOID_JOINTS):
            q0, q1 = self.q[j, k0], self.q[j, k0 + 1]
            q = (q0 + (q1 - q0) * a).astype(F32)
            q = (q / F32(np.sqrt(F32(F32(F32(q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3])))).astype(F32)
            if parent < 0:
                off = np.asarray(bp, dtype=F32)
            else:
                off = (np.asarray(bp, dtype=F32) - np.asarray(HUMANOID_JOINTS[parent][2], dtype=F32)).astype(F32)
            local = mat_mul(_quat_to_mat(q), mat_translate(*off))
            g = local if parent < 0 else mat_mul(local, glob[parent])
            glob.append(g)
            inv_bind = mat_translate(*(-np.asarray(bp, dtype=F32)))
            out[j] = mat_mul(inv_bind, g)
        return out


def humanoid_model(sc: Scene, seed: int, tex_size: int = 512) -> int:
    mesh = humanoid_mesh(seed)
    ml = build_meshlets(mesh)
    # skinned bounds must hold the deformed meshlet around the culling bone
    ml.cull[:, 3] = (ml.cull[:, 3] * F32(1.5) + F32(0.25)).astype(F32)
    tex = sc.add_texture(value_noise_texture(tex_size, tex_size, seed * 17 + 3))
    mat = sc.add_material(tex, 0xFFFFFFFF, 16.0)
    proxies = []
    for part, bone in HUMANOID_PROXIES:
        a, b, r, _ = HUMANOID_PARTS[part]
        proxies.append((a, b, r, bone))
    return sc.add_model(Model([ml], [mat], bone_count=len(HUMANOID_JOINTS), proxies=proxies))


def ground_model(sc: Scene, seed: int, n: int = 64, half: float = 16.0, center=(0.0, 0.0, 8.0), tex_size: int = 512,
                 lightmap: int | None = None) -> int:
    cx, cy, cz = (F32(c) for c in center)
    xs = (np.arange(n + 1, dtype=F32) / F32(n) * F32(2 * half) - F32(half)).astype(F32)
    pos, nrm, uv, tris = [], [], [], []
    for j in range(n + 1):
        for i in range(n + 1):
            pos.append([F32(cx + xs[i]), cy, F32(cz + xs[j])])
            nrm.append([0.0, 1.0, 0.0])
            uv.append([F32(i) / F32(8), F32(j) / F32(8)])
    for j in range(n):
        for i in range(n):
            a, b, c, d = j * (n + 1) + i, j * (n + 1) + i + 1, (j + 1) * (n + 1) + i + 1, (j + 1) * (n + 1) + i
            tris += [[a, b, c], [a, c, d]]
    pos, nrm = np.array(pos, dtype=F32), np.array(nrm, dtype=F32)
    mesh = RawMesh(pos, nrm, np.array(uv, dtype=F32), _orient(pos, nrm, np.array(tris)))
    tex = sc.add_texture(value_noise_texture(tex_size, tex_size, seed * 19 + 5))
    mat = sc.add_material(tex, 0xFFFFFFFF, 32.0)
    return sc.add_model(Model([build_meshlets(mesh)], [mat]))


def skinned_characters_scene(width=1920, height=1080, seed=2001, n_chars=8, n_lights=4, tex_size=512, frames=1,
                             ground_quads=64, time0=0.0, views=None) -> Scene:
    """Skinned humanoids on a ground plane, lit by point lights above them; one capsule proxy per
    head, torso, upper/lower arm and thigh/shin."""
    rng = Pcg32(seed)
    sc = Scene()
    ground = ground_model(sc, seed, n=ground_quads)
    chars, anims = [], []
    for c in range(n_chars):
        chars.append(humanoid_model(sc, seed * 97 + c, tex_size))
        anims.append(HumanoidAnim(seed * 89 + c))
    place = []
    for c in range(n_chars):
        col, row = c % 4, c // 4
        x = F32(F32(-3.0 + 2.0 * col) + rng.uniform(-0.3, 0.3))
        z = F32(F32(5.0 + 3.0 * row) + rng.uniform(-0.3, 0.3))
        yaw = rng.uniform(0.0, 6.28318530717959)
        place.append(mat_mul(mat_rot_y(yaw), mat_translate(x, F32(0.0), z)))
    lights = []
    for l in range(n_lights):
        lp = (rng.uniform(-6.0, 6.0), rng.uniform(5.0, 7.0), rng.uniform(3.0, 11.0))
        col = (rng.uniform(0.6, 1.0), rng.uniform(0.6, 1.0), rng.uniform(0.6, 1.0))
        lights.append((lp, col[0], col[1], col[2], F32(1.0), F32(14.0)))
    if views is None:
        views = [(width, height, (0.0, 1.7, 0.0), (0.0, 1.0, 8.0), F32(time0 + fi / max(frames, 1)) % F32(1.0))
                 for fi in range(frames)]
    for vw, vh, cpos, tgt, t in views:
        fr = _camera_frame(vw, vh, cam_pos=cpos, target=tgt)
        fr.ambient = np.array([0.15, 0.15, 0.17], dtype=F32)
        fr.point_lights = list(lights)
        insts = [(ground, mat_identity(), None)]
        for c in range(n_chars):
            insts.append((chars[c], place[c], anims[c].pose(t)))
        fr.instances = insts
        sc.frames.append(fr)
    return sc


def config2(width=1920, height=1080, seed=2001) -> Scene:
    """Skinned characters at 1920x1080 (rendered with 2x MSAA): eight ~6k-triangle humanoids on
    a 22-joint skeleton, ground of 64x64 quads, four point lights, 512x512 textures."""
    return skinned_characters_scene(width, height, seed)


# ------------------------------------------------------------------ edge-case variety scene
def variety_scene(width=320, height=200, seed=4001, n_objects=20, n_lights=18, n_dir=2, near_camera=True,
                  clear=1) -> Scene:
    """Parity scene for the less common branches: camera inside the object field (near-plane
    clipping), untextured and emissive materials, NPOT textures with non-negative UVs,
    directional lights, more point lights than the per-tile cap of 16, optional no-clear."""
    rng = Pcg32(seed)
    sc = Scene()
    sphere_ml = build_meshlets(uv_sphere(16, 8, 0.5))
    cube_ml = build_meshlets(box((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)))
    # NPOT bilinear reads are only defined for texel coordinates >= 0 in the reference
    # (sofren2.c:5594-5600), so the NPOT material's UVs stay inside [0.1, 0.9]
    inner = uv_sphere(16, 8, 0.5)
    inner.uv = (inner.uv * F32(0.8) + F32(0.1)).astype(F32)
    sphere_npot_ml = build_meshlets(inner)
    tex_pot = sc.add_texture(value_noise_texture(64, 64, seed + 1, lattice=8))
    tex_npot = sc.add_texture(value_noise_texture(48, 40, seed + 2, lattice=8))
    mats = [sc.add_material(tex_pot, 0xFFFFFFFF, 16.0), sc.add_material(tex_npot, 0xFFC08040, 8.0),
            sc.add_material(-1, 0xFF80C0FF, 4.0), sc.add_material(tex_pot, 0xFFFFFFFF, -1.5),
            sc.add_material(-1, 0xFFFFFFFF, 64.0)]
    models = []
    for k, mat in enumerate(mats):
        models.append(sc.add_model(Model([sphere_npot_ml if k == 1 else sphere_ml], [mat], proxies=[((0, 0, 0), (0, 0, 0), 0.45, 0xFFFFFFFF)])))
        if k != 1:
            models.append(sc.add_model(Model([cube_ml], [mat], proxies=[((0, -0.2, 0), (0, 0.2, 0), 0.4, 0xFFFFFFFF)])))
    insts = []
    zc = 2.0 if near_camera else 8.0
    for i in range(n_objects):
        mi = models[i % len(models)]
        p = (rng.uniform(-3, 3), rng.uniform(-2, 2), F32(zc + rng.uniform(-2.0, 4.0)))
        s = rng.uniform(0.5, 1.8)
        tr = mat_mul(mat_mul(mat_scale(s), mat_rot_y(rng.uniform(0, 6.28318530717959))), mat_translate(*p))
        insts.append((mi, tr, None))
    lights = []
    for l in range(n_lights):
        lp = (rng.uniform(-4, 4), F32(rng.uniform(9.0, 11.0)), rng.uniform(3.0, 9.0))
        lights.append((lp, rng.uniform(0.3, 1.0), rng.uniform(0.3, 1.0), rng.uniform(0.3, 1.0), F32(0.8), rng.uniform(12.0, 20.0)))
    fr = _camera_frame(width, height)
    fr.ambient = np.array([0.12, 0.1, 0.1], dtype=F32)
    fr.point_lights = lights
    fr.dir_lights = [((rng.uniform(-1, 1), F32(-1.0), rng.uniform(-1, 1)), F32(0.8), F32(0.8), F32(0.7), F32(0.6))
                     for _ in range(n_dir)]
    fr.clear = clear
    fr.instances = insts
    sc.frames.append(fr)
    return sc


# ------------------------------------------------------------------ lightmapped atrium
class _QuadMesh:
    """Accumulates quads (4 verts, 2 tris) with flat normals, UVs and a lightmap chart each."""

    def __init__(self, lm_size: int, chart_base: list):
        self.pos, self.nrm, self.uv, self.luv, self.tris = [], [], [], [], []
        self.lm_size, self.chart = lm_size, chart_base   # shared [next chart index]

    def quad(self, p0, p1, p2, p3, n, uv_scale=1.0):
        base = len(self.pos)
        c = self.chart[0]
        self.chart[0] += 1
        cols = self.lm_size // 2
        cx, cy = (c % cols) * 2, (c // cols) * 2
        inv = F32(1.0 / self.lm_size)
        corners = ((0, 0), (0, 1), (1, 1), (1, 0))
        for (p, (i, j)) in zip((p0, p1, p2, p3), corners):
            self.pos.append(p)
            self.nrm.append(n)
            self.uv.append([F32(i) * F32(uv_scale), F32(j) * F32(uv_scale)])
            self.luv.append([F32(F32(cx + i) + F32(0.5)) * inv, F32(F32(cy + j) + F32(0.5)) * inv])
        self.tris += [[base, base + 1, base + 2], [base, base + 2, base + 3]]

    def box(self, lo, hi, uv_scale=1.0):
        lo, hi = np.asarray(lo, dtype=F32), np.asarray(hi, dtype=F32)
        for ax in range(3):
            for sgn in (-1, 1):
                ua, va = [a for a in range(3) if a != ax]
                n = np.zeros(3, dtype=F32); n[ax] = F32(sgn)
                pts = []
                for (cu, cv) in ((0, 0), (0, 1), (1, 1), (1, 0)):
                    p = np.zeros(3, dtype=F32)
                    p[ax] = hi[ax] if sgn > 0 else lo[ax]
                    p[ua] = hi[ua] if cu else lo[ua]
                    p[va] = hi[va] if cv else lo[va]
                    pts.append(p)
                e1, e2 = (pts[1] - pts[0]).astype(F32), (pts[2] - pts[0]).astype(F32)
                if _dot3(_cross3(e1, e2), n) < 0:
                    pts = [pts[0], pts[3], pts[2], pts[1]]
                self.quad(*pts, n, uv_scale)

    def raw(self) -> RawMesh:
        pos = np.array(self.pos, dtype=F32).reshape(-1, 3)
        return RawMesh(pos, np.array(self.nrm, dtype=F32), np.array(self.uv, dtype=F32), np.array(self.tris).reshape(-1, 3),
                       luv=np.array(self.luv, dtype=F32))


_ATRIUM_GEOMETRY: dict = {}


def _atrium_geometry(lm_size, nx, nz, levels, arch_segments, n_tex, floor_quads):
    """The atrium's static meshes, [(texture group, Meshlets)], and its lightmap chart count.
    Depends on the layout parameters only, so scenes of one layout share it (memoised)."""
    key = (lm_size, nx, nz, levels, arch_segments, n_tex, tuple(floor_quads))
    if key in _ATRIUM_GEOMETRY:
        return _ATRIUM_GEOMETRY[key]
    chart = [0]
    groups = [_QuadMesh(lm_size, chart) for _ in range(n_tex)]
    x0, x1, z0, z1, height_m = -15.0, 15.0, 4.0, 19.0, 15.0
    fq = _QuadMesh(lm_size, chart)
    fx, fz = floor_quads
    for j in range(fz):
        for i in range(fx):
            ax, bx = F32(x0 + (x1 - x0) * i / fx), F32(x0 + (x1 - x0) * (i + 1) / fx)
            az, bz = F32(z0 + (z1 - z0) * j / fz), F32(z0 + (z1 - z0) * (j + 1) / fz)
            fq.quad(np.array([ax, 0, az], F32), np.array([ax, 0, bz], F32), np.array([bx, 0, bz], F32),
                    np.array([bx, 0, az], F32), np.array([0, 1, 0], F32), 0.25)
    wq = _QuadMesh(lm_size, chart)
    wy = max(1, fz)
    for j in range(wy):
        for i in range(fx):
            ax, bx = F32(x0 + (x1 - x0) * i / fx), F32(x0 + (x1 - x0) * (i + 1) / fx)
            ay, by = F32(height_m * j / wy), F32(height_m * (j + 1) / wy)
            wq.quad(np.array([ax, ay, z1], F32), np.array([ax, by, z1], F32), np.array([bx, by, z1], F32),
                    np.array([bx, ay, z1], F32), np.array([0, 0, -1], F32), 0.25)
    dx, dz = (x1 - x0) / nx, (z1 - z0) / nz
    lvl_h = height_m / levels
    pw = 0.18
    for lv in range(levels):
        yb = lv * lvl_h
        ph = lvl_h * 0.55
        for iz in range(nz):
            for ix in range(nx):
                g = groups[(ix + iz * nx + lv * 7) % n_tex]
                cxp, czp = x0 + dx * (ix + 0.5), z0 + dz * (iz + 0.5)
                g.box((cxp - pw, yb, czp - pw), (cxp + pw, yb + ph, czp + pw))
                for (ddx, ddz) in ((1, 0), (0, 1)):
                    if (ddx and ix == nx - 1) or (ddz and iz == nz - 1):
                        continue
                    span = dx if ddx else dz
                    rad = span * 0.5
                    for sgi in range(arch_segments):
                        a0 = F32(_PI * sgi / arch_segments)
                        a1 = F32(_PI * (sgi + 1) / arch_segments)
                        am = F32((a0 + a1) * F32(0.5))
                        ca, sa = float(dcos(am)), float(dsin(am))
                        cx_ = cxp + ddx * (rad - rad * ca)
                        cz_ = czp + ddz * (rad - rad * ca)
                        cy_ = yb + ph + rad * sa
                        hl = rad * np.pi / arch_segments * 0.5 + 0.01
                        ext = (hl if ddx else 0.08, 0.06, hl if ddz else 0.08)
                        g.box((cx_ - ext[0], cy_ - ext[1], cz_ - ext[2]), (cx_ + ext[0], cy_ + ext[1], cz_ + ext[2]))
    built = [(t, build_meshlets(g.raw())) for t, g in enumerate(groups + [fq, wq]) if g.tris]
    _ATRIUM_GEOMETRY[key] = (built, chart[0])
    return _ATRIUM_GEOMETRY[key]


def atrium_scene(width=1920, height=1080, seed=3001, nx=20, nz=10, levels=3, arch_segments=16, n_tex=25,
                 tex_size=1024, lm_size=1024, n_lights=16, n_chars=4, char_tex=512, floor_quads=(120, 60), frames=1,
                 views=None) -> Scene:
    """An atrium of pillars and semicircular arches (boxes, arch_segments per arch) on `levels`
    floors of an nx x nz grid, floor and walls as quad grids; every static quad owns a 2x2 texel
    chart in one lightmap page holding per-vertex baked colours uniform in [0,1]^3.  Point
    lights sit under the roof with a radius that covers the whole atrium, and skinned humanoids
    stand on the floor."""
    rng = Pcg32(seed)
    sc = Scene()
    built, n_chart = _atrium_geometry(lm_size, nx, nz, levels, arch_segments, n_tex, floor_quads)
    chart = [n_chart]
    assert chart[0] * 4 <= lm_size * lm_size, "lightmap page too small for the quad charts"
    lm = np.full((lm_size, lm_size), 0xFF000000, dtype=np.uint32)
    cols_rgb = np.zeros((chart[0] * 4, 3), dtype=np.uint32)
    for k in range(chart[0] * 4):
        cols_rgb[k] = [rng.next_u32() >> 24, rng.next_u32() >> 24, rng.next_u32() >> 24]
    cols = lm_size // 2
    ci = np.arange(chart[0])
    cx, cy = (ci % cols) * 2, (ci // cols) * 2
    for q, (i, j) in enumerate(((0, 0), (0, 1), (1, 1), (1, 0))):
        c = cols_rgb[q::4]
        lm[cy + j, cx + i] = 0xFF000000 | (c[:, 0] << 16) | (c[:, 1] << 8) | c[:, 2]
    lm_tex = sc.add_texture(lm)
    tex_ids = [sc.add_texture(value_noise_texture(tex_size, tex_size, seed * 31 + t)) for t in range(n_tex)]
    meshes, mats = [], []
    for t, ms in built:
        meshes.append(ms)
        mats.append(sc.add_material(tex_ids[t % n_tex], 0xFFFFFFFF, 16.0))
    atrium = sc.add_model(Model(meshes, mats, lightmaps=[lm_tex], lightmap_pages=[0] * len(meshes)))
    chars, anims = [], []
    for c in range(n_chars):
        chars.append(humanoid_model(sc, seed * 97 + c, char_tex))
        anims.append(HumanoidAnim(seed * 89 + c))
    place = []
    for c in range(n_chars):
        x = F32(F32(-1.5 + 1.0 * c) + rng.uniform(-0.2, 0.2))
        z = F32(rng.uniform(5.5, 7.0))
        place.append(mat_mul(mat_rot_y(rng.uniform(0.0, 6.28318530717959)), mat_translate(x, F32(0.0), z)))
    lights = []
    for l in range(n_lights):
        lp = (rng.uniform(-12.0, 12.0), rng.uniform(13.0, 14.5), rng.uniform(6.0, 17.0))
        lights.append((lp, rng.uniform(0.6, 1.0), rng.uniform(0.6, 1.0), rng.uniform(0.6, 1.0), F32(0.5), F32(60.0)))
    if views is None:
        views = [(width, height, (0.0, 1.7, 0.5), (0.0, 3.0, 12.0), F32(fi / max(frames, 1))) for fi in range(frames)]
    for vw, vh, cpos, tgt, t in views:
        fr = _camera_frame(vw, vh, cam_pos=cpos, target=tgt)
        fr.ambient = np.array([0.1, 0.1, 0.1], dtype=F32)
        fr.point_lights = list(lights)
        fr.instances = [(atrium, mat_identity(), None)] + [(chars[c], place[c], anims[c].pose(t)) for c in range(n_chars)]
        sc.frames.append(fr)
    return sc


MULTIVIEW_SIZES = ((320, 180), (640, 360), (1280, 720), (1920, 1080), (2560, 1440))


def config4(seed=4001, n_views=96, n_scenes=6, quick=False) -> tuple[list[Scene], list[tuple[int, int, int]]]:
    """Batched multi-view workload: n_views views over n_scenes resident scenes (half of the
    skinned-characters type, half of the atrium type, each with its own seed).  Each view draws
    its resolution from MULTIVIEW_SIZES, its MSAA from (1, 2, 4), a seeded camera looking into the
    scene and an animation time in [0, 1).  Returns (scenes, [(scene index, frame index, samples)]),
    view k being frame k // n_scenes of scene k % n_scenes.  quick=True shrinks the atrium type
    (fewer textures and floor quads) for CPU-side tests."""
    rng = Pcg32(seed)
    per_scene: list[list] = [[] for _ in range(n_scenes)]
    out_views = []
    for k in range(n_views):
        si = k % n_scenes
        w, h = MULTIVIEW_SIZES[rng.next_u32() % len(MULTIVIEW_SIZES)]
        S = (1, 2, 4)[rng.next_u32() % 3]
        t = F32(rng.uniform(0.0, 1.0))
        if si < n_scenes // 2:   # skinned characters: characters at z 5..8, x -3..3
            cpos = (rng.uniform(-4.0, 4.0), rng.uniform(1.2, 2.6), rng.uniform(-1.0, 1.5))
            tgt = (rng.uniform(-2.0, 2.0), rng.uniform(0.6, 1.4), rng.uniform(6.0, 9.0))
        else:                    # atrium: floor 30 x 15 m from z ~1, characters near z 6
            cpos = (rng.uniform(-5.0, 5.0), rng.uniform(1.5, 4.0), rng.uniform(0.2, 2.5))
            tgt = (rng.uniform(-4.0, 4.0), rng.uniform(1.0, 5.0), rng.uniform(9.0, 15.0))
        out_views.append((si, len(per_scene[si]), S))
        per_scene[si].append((w, h, cpos, tgt, t))
    scenes = []
    for si in range(n_scenes):
        if si < n_scenes // 2:
            scenes.append(skinned_characters_scene(seed=2001 + 10 * si, views=per_scene[si]))
        elif quick:
            scenes.append(atrium_scene(seed=3001 + 10 * si, nx=10, nz=5, levels=2, n_tex=4, tex_size=128, lm_size=512,
                                       char_tex=64, floor_quads=(30, 15), views=per_scene[si]))
        else:
            scenes.append(atrium_scene(seed=3001 + 10 * si, views=per_scene[si]))
    return scenes, out_views


def config5(seed=5001, n_scenes=16, frames_per_scene=24, quick=False) -> tuple[list[Scene], list[int]]:
    """Served-rendering scenes: n_scenes resident scenes, half of the skinned-characters type
    (eight humanoids, sixteen point lights, rendered at 2x MSAA) and half of the atrium type (the
    config-3 layout with per-scene textures, lightmap colours, lights and characters, rendered at
    4x MSAA).  Each scene holds a pool of frames_per_scene request frames: a seeded camera, a
    resolution from MULTIVIEW_SIZES and an animation time in [0, 1).  Returns (scenes, MSAA per
    scene).  quick=True shrinks the atrium type for CPU-side tests."""
    rng = Pcg32(seed)
    scenes_out, samples = [], []
    for si in range(n_scenes):
        views = []
        skinned = si < n_scenes // 2
        for _ in range(frames_per_scene):
            w, h = MULTIVIEW_SIZES[rng.next_u32() % len(MULTIVIEW_SIZES)]
            t = F32(rng.uniform(0.0, 1.0))
            if skinned:
                cpos = (rng.uniform(-4.0, 4.0), rng.uniform(1.2, 2.6), rng.uniform(-1.0, 1.5))
                tgt = (rng.uniform(-2.0, 2.0), rng.uniform(0.6, 1.4), rng.uniform(6.0, 9.0))
            else:
                cpos = (rng.uniform(-5.0, 5.0), rng.uniform(1.5, 4.0), rng.uniform(0.2, 2.5))
                tgt = (rng.uniform(-4.0, 4.0), rng.uniform(1.0, 5.0), rng.uniform(9.0, 15.0))
            views.append((w, h, cpos, tgt, t))
        if skinned:
            scenes_out.append(skinned_characters_scene(seed=seed + 10 * si, n_lights=16, views=views))
            samples.append(2)
        elif quick:
            scenes_out.append(atrium_scene(seed=seed + 10 * si, nx=10, nz=5, levels=2, n_tex=4, tex_size=128, lm_size=512,
                                           char_tex=64, floor_quads=(30, 15), views=views))
            samples.append(4)
        else:
            scenes_out.append(atrium_scene(seed=seed + 10 * si, views=views))
            samples.append(4)
    return scenes_out, samples


def _quat(axis, ang):
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    h = 0.5 * ang
    return np.array([*(axis * np.sin(h)), np.cos(h)], np.float32)


def _trs_matrix(t, q, sc):
    x, y, z, w = [float(v) for v in q]
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y + w * z), 2 * (x * z - w * y), 0],
                  [2 * (x * y - w * z), 1 - 2 * (x * x + z * z), 2 * (y * z + w * x), 0],
                  [2 * (x * z + w * y), 2 * (y * z - w * x), 1 - 2 * (x * x + y * y), 0], [0, 0, 0, 1]])
    m = np.diag([sc[0], sc[1], sc[2], 1.0]) @ r
    m[3, :3] += np.asarray(t)
    return m.astype(np.float32)


def pose_rig(seed=6001, n_bones=22, n_keys=30) -> dict:
    """A seeded skeleton with two animations, in the layout of sft_bone / sft_animation
    (sofren2.c:1000-1049): a random bone tree, rest TRS and bind matrices, animation 0 rotating
    every bone (30 linear keys, with sign flips and near-identical neighbours to reach both slerp
    branches) plus a root translation and a stepped scale, animation 1 with stepped rotations of
    half the bones and two channels driving the same node and path (the later one must win)."""
    rng = np.random.default_rng(seed)
    bones = []
    for b in range(n_bones):
        parent = -1 if b == 0 else int(rng.integers(0, b))
        t = rng.uniform(-0.3, 0.3, 3).astype(np.float32)
        q = _quat(rng.normal(size=3), rng.uniform(-0.6, 0.6))
        sc = rng.uniform(0.9, 1.1, 3).astype(np.float32)
        inv = _trs_matrix(rng.uniform(-1, 1, 3), _quat(rng.normal(size=3), rng.uniform(-3, 3)), rng.uniform(0.8, 1.2, 3))
        bones.append(dict(parent=parent, base_t=t, base_r=q, base_s=sc, local_bind=_trs_matrix(t, q, sc), inverse_bind=inv))

    def keys(n, duration):
        return np.sort(np.concatenate([[0.0], rng.uniform(0, duration, n - 2), [duration]])).astype(np.float32)

    def rot_track(n, duration):
        out = np.zeros((n, 4), np.float32)
        axis = rng.normal(size=3)
        for k in range(n):
            q = _quat(axis + 0.2 * rng.normal(size=3), rng.uniform(-2.5, 2.5))
            if k % 7 == 3:
                q = -q                      # same rotation, opposite sign: dot < 0
            if k % 11 == 5 and k > 0:
                q = out[k - 1] + np.float32(1e-4)   # near-identical neighbour: lerp branch
                q = (q / np.linalg.norm(q)).astype(np.float32)
            out[k] = q
        return keys(n, duration), out

    anims = []
    samplers, channels = [], []
    for b in range(n_bones):
        ins, outs = rot_track(n_keys, 1.0)
        samplers.append((ins, outs, 0)); channels.append((len(samplers) - 1, b, 1))
    t_out = np.zeros((n_keys, 4), np.float32); t_out[:, :3] = rng.uniform(-0.5, 0.5, (n_keys, 3))
    samplers.append((keys(n_keys, 1.0), t_out, 0)); channels.append((len(samplers) - 1, 0, 0))
    s_out = np.zeros((8, 4), np.float32); s_out[:, :3] = rng.uniform(0.8, 1.2, (8, 3))
    samplers.append((keys(8, 1.0), s_out, 1)); channels.append((len(samplers) - 1, 5, 2))
    anims.append(dict(duration=np.float32(1.0), samplers=samplers, channels=channels))
    samplers, channels = [], []
    for b in range(0, n_bones, 2):
        ins, outs = rot_track(12, 0.8)
        samplers.append((ins, outs, 1)); channels.append((len(samplers) - 1, b, 1))
    ins, outs = rot_track(12, 0.8)
    samplers.append((ins, outs, 0)); channels.append((len(samplers) - 1, 2, 1))   # second channel on bone 2
    channels.append((0, n_bones + 3, 1))                                            # node out of range: skipped
    anims.append(dict(duration=np.float32(0.8), samplers=samplers, channels=channels))
    return dict(bones=bones, anims=anims)


def pose_requests(rig: dict, n: int, seed: int = 7) -> list[tuple[int, float]]:
    """(animation, time) requests: times inside, before and after the clip (fmodf wraps them),
    exactly on keyframes, and a few with an out-of-range animation index."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        a = int(rng.integers(0, len(rig["anims"])))
        kind = k % 6
        if kind == 0:
            t = float(rng.uniform(0, 1))
        elif kind == 1:
            t = float(rng.uniform(1, 5))
        elif kind == 2:
            t = float(rng.uniform(-1, 0))
        elif kind == 3:
            ins = rig["anims"][a]["samplers"][0][0]
            t = float(ins[int(rng.integers(0, len(ins)))])
        elif kind == 4:
            t = 0.0
        else:
            a, t = (-1 if k % 12 == 5 else 7), 0.5
        out.append((a, np.float32(t)))
    return out


def config3(width=1920, height=1080, seed=3001) -> Scene:
    """Large static scene (rendered with 4x MSAA): about 262k triangles of boxes and
    semicircular arches forming a 30x15x15 m atrium, 25 textures of 1024x1024, a baked
    lightmap page, four skinned characters, sixteen point lights covering the floor."""
    return atrium_scene(width, height, seed)


RAY_RECORD = np.dtype([("T", "<f4", (16,)), ("o", "<f4", (3,)), ("d", "<f4", (3,)), ("max_dist", "<f4"), ("model", "<i4")])


def ray_batch(sc: Scene, n: int, seed: int = 6001, frame: int = 0) -> np.ndarray:
    """n ray queries (sftg_ray records; `model` is the scene's model index) against the instances
    of one frame: origins scattered around the camera, 70% aimed at points of a model's bounds
    as sft_raycast_instance places the model (transform rows 0-2, no translation), 20% random
    directions, 10% along coordinate axes; distance limit 1000, 10% a short one."""
    rng = np.random.default_rng(seed)
    fr = sc.frames[frame]
    insts = [(mi, np.asarray(T, np.float32).reshape(4, 4)) for mi, T, _ in fr.instances]
    lo, hi = {}, {}
    for mi, _ in insts:
        if mi not in lo:
            pos = np.concatenate([ms.attr.reshape(ms.n, 10, 64)[:, 0:3].transpose(0, 2, 1).reshape(-1, 3) for ms in sc.models[mi].meshes])
            lo[mi], hi[mi] = pos.min(0), pos.max(0)
    pick = rng.integers(0, len(insts), n)
    out = np.zeros(n, RAY_RECORD)
    Ts = np.stack([T for _, T in insts])
    out["T"] = Ts[pick].reshape(n, 16)
    out["model"] = np.array([mi for mi, _ in insts], np.int32)[pick]
    o = (np.asarray(fr.cam_pos, np.float32) + rng.normal(0, 1.5, (n, 3))).astype(np.float32)
    out["o"] = o
    L = np.stack([lo[mi] for mi, _ in insts])[pick]
    Hh = np.stack([hi[mi] for mi, _ in insts])[pick]
    p = (L + rng.random((n, 3)) * (Hh - L)).astype(np.float32)
    aimed = np.einsum("nj,njk->nk", p, Ts[pick][:, :3, :3]).astype(np.float32) - o
    rand_d = rng.normal(0, 1, (n, 3)).astype(np.float32)
    axis_d = np.zeros((n, 3), np.float32)
    axis_d[np.arange(n), rng.integers(0, 3, n)] = rng.choice([-1.0, 1.0], n)
    kind = rng.random(n)
    d = np.where((kind < 0.7)[:, None], aimed, np.where((kind < 0.9)[:, None], rand_d, axis_d))
    out["d"] = d.astype(np.float32)
    out["max_dist"] = np.where(rng.random(n) < 0.1, rng.uniform(0.5, 3.0, n), 1000.0).astype(np.float32)
    return out
