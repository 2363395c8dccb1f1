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
