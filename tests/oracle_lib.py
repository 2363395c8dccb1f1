"""ctypes access to the CPU oracle (oracle/sft_oracle.c) for tests and the CPU baseline.

Test infrastructure only: the shipped library never loads this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

from oracle_io import read_dump

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "libsft_oracle.so")
REF_DIR = os.path.join(ROOT, "oracle", "_ref")


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)
    return ORACLE_SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        L = C.CDLL(ORACLE_SO)
        L.sfto_open.restype, L.sfto_open.argtypes = C.c_void_p, [C.c_void_p, C.c_uint64]
        L.sfto_render.restype = C.c_int
        L.sfto_render.argtypes = [C.c_void_p, C.c_uint32, C.c_int, C.c_int, C.c_char_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p]
        L.sfto_close.restype, L.sfto_close.argtypes = None, [C.c_void_p]
        L.sfto_set_debug_mode.restype, L.sfto_set_debug_mode.argtypes = C.c_int, [C.c_void_p, C.c_int]
        _lib = L
    return _lib


class Oracle:
    def __init__(self, blob: bytes):
        self._buf = np.frombuffer(blob, dtype=np.uint8)
        self.h = lib().sfto_open(self._buf.ctypes.data_as(C.c_void_p), len(blob))
        if not self.h:
            raise RuntimeError("oracle rejected the scene blob")

    def model_blas(self, mi: int) -> tuple[bytes, int]:
        """(node images, root index) of model mi's BLAS, built by the oracle's restated builder."""
        L = lib()
        L.sfto_model_blas.restype = C.c_int
        L.sfto_model_blas.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]
        root = C.c_uint32(0)
        n = L.sfto_model_blas(self.h, mi, None, 0, C.byref(root))
        buf = np.zeros(max(1, n) * 256, np.uint8)
        L.sfto_model_blas(self.h, mi, buf.ctypes.data_as(C.c_void_p), n, C.byref(root))
        return buf[: n * 256].tobytes(), int(root.value)

    def shadow_fp64(self, frame: int, samples: int) -> dict:
        """The frame's capsule shadows evaluated in double beside the FP32 restatement (which is
        the reference's arithmetic): largest and mean |FP32 - FP64| shadow intensity, the number
        of pixel x light evaluations and how many differ by more than 1e-5."""
        L = lib()
        L.sfto_shadow_fp64.restype = C.c_int
        L.sfto_shadow_fp64.argtypes = [C.c_void_p, C.c_uint32, C.c_int, C.c_void_p]
        out = np.zeros(4, np.float64)
        if L.sfto_shadow_fp64(self.h, frame, samples, out.ctypes.data_as(C.c_void_p)) != 0:
            raise RuntimeError("oracle FP64 shadow evaluation failed")
        return {"max": float(out[0]), "mean": float(out[1]), "n": int(out[2]), "over_1e-5": int(out[3])}

    def blas_rebuild(self, mi: int, reps: int = 1) -> int:
        """Builds model mi's BLAS again `reps` times with the oracle's restated builder (timing)."""
        L = lib()
        L.sfto_blas_rebuild.restype = C.c_int
        L.sfto_blas_rebuild.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32]
        return int(L.sfto_blas_rebuild(self.h, mi, reps))

    def raycast(self, rays: np.ndarray) -> np.ndarray:
        """The oracle's sft_raycast_instance restatement for each RAY_DTYPE record."""
        L = lib()
        L.sfto_raycast.restype = C.c_int
        L.sfto_raycast.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        out = np.zeros(len(r), HIT_DTYPE)
        if L.sfto_raycast(self.h, r.ctypes.data_as(C.c_void_p), len(r), out.ctypes.data_as(C.c_void_p)) != 0:
            raise ValueError("ray with a bad model index")
        return out

    def set_debug_mode(self, mode: int) -> None:
        if lib().sfto_set_debug_mode(self.h, mode) != 0:
            raise ValueError(f"bad debug mode {mode}")

    def close(self):
        if self.h:
            lib().sfto_close(self.h)
            self.h = None

    def render_dump(self, frame: int, samples: int, threads: int = 1, shadow: bool = False) -> dict:
        """Renders one frame and returns its dump sections (plus 'ns', 'invalid_packets', 'shadow')."""
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "o.dump")
            ns, inv = np.zeros(1, np.uint64), np.zeros(1, np.uint32)
            rc = lib().sfto_render(self.h, frame, samples, threads, path.encode(), None, None,
                                   ns.ctypes.data_as(C.c_void_p), inv.ctypes.data_as(C.c_void_p))
            if rc != 0:
                raise RuntimeError(f"oracle render failed ({rc})")
            frames = read_dump(path)
        out = frames[-1]
        out["blas"] = frames[0].get("blas", [])
        out["ns"] = int(ns[0])
        out["invalid_packets"] = int(inv[0])
        return out

    def render_color(self, frame: int, samples: int, width: int, height: int, threads: int = 1,
                     shadow: bool = False) -> tuple[np.ndarray, int, np.ndarray | None]:
        color = np.zeros(width * height, np.uint32)
        ns = np.zeros(1, np.uint64)
        sh = np.zeros(width * height * 16, np.float32) if shadow else None
        rc = lib().sfto_render(self.h, frame, samples, threads, None, color.ctypes.data_as(C.c_void_p),
                               None if sh is None else sh.ctypes.data_as(C.c_void_p), ns.ctypes.data_as(C.c_void_p), None)
        if rc != 0:
            raise RuntimeError(f"oracle render failed ({rc})")
        return color, int(ns[0]), sh


def qsf_bytes(scene, mi: int, blas: bytes, blas_root: int) -> bytes:
    """Model mi of a scenes.Scene written in the reference's QSF2 layout (sft_model_load_qsf,
    sofren2.c:7816-7967): textures (each becomes a white material of shininess 2), lightmap
    pages, the model header, per mesh its meshlets (positions, then normals / UVs / lightmap
    UVs), flat indices, bounding spheres, boxes and cones, then the meshlet-to-mesh table and
    the BLAS nodes."""
    import struct
    m = scene.models[mi]
    tex_ids = sorted({scene.materials[mat][0] for mat in m.materials if mat >= 0 and scene.materials[mat][0] >= 0})
    tex_pos = {t: i for i, t in enumerate(tex_ids)}
    out = [b"QSF2", struct.pack("<IQ", 2, 0), struct.pack("<I", len(tex_ids))]
    for t in tex_ids:
        tx = scene.textures[t]
        out.append(struct.pack("<II", tx.shape[1], tx.shape[0]) + tx.astype("<u4").tobytes())
    out.append(struct.pack("<I", len(m.lightmaps)))
    for t in m.lightmaps:
        tx = scene.textures[t]
        out.append(struct.pack("<II", tx.shape[1], tx.shape[0]) + tx.astype("<u4").tobytes())
    total = sum(ms.n for ms in m.meshes)
    out.append(struct.pack("<IIII", len(m.meshes), total, len(blas) // 256, blas_root))
    first = 0
    for ms, mat, page in zip(m.meshes, m.materials, m.lightmap_pages):
        tex = scene.materials[mat][0] if mat >= 0 else -1
        out.append(struct.pack("<IIII", ms.n, first, tex_pos.get(tex, 0xFFFFFFFF), page))
        attr = ms.attr.reshape(ms.n, 10, 64).astype("<f4")
        out.append(attr[:, 0:3].tobytes())                     # sft_meshlet: x y z
        out.append(attr[:, 3:10].tobytes())                    # attribs: nx ny nz u v lu lv
        flat = np.zeros((ms.n, 128, 3), np.uint8)
        ind = ms.inds.reshape(ms.n, 16, 32)
        for k in range(3):
            flat[:, :, k] = ind[:, :, 8 * k:8 * k + 8].reshape(ms.n, 128)
        out.append(flat.tobytes())
        cull = ms.cull.reshape(ms.n, 8).astype("<f4")
        pos = attr[:, 0:3]
        for k in range(4):                                     # sphere centre x y z, radius
            out.append(np.ascontiguousarray(cull[:, k]).tobytes())
        out.append(pos.min(axis=2).T.copy().tobytes())         # box min x y z
        out.append(pos.max(axis=2).T.copy().tobytes())         # box max x y z
        for k in range(4, 8):                                  # cone axis x y z, cutoff
            out.append(np.ascontiguousarray(cull[:, k]).tobytes())
        first += ms.n
    out.append(np.concatenate([np.full(ms.n, i, "<u2") for i, ms in enumerate(m.meshes)]).tobytes())
    out.append(blas)
    return b"".join(out)


def pose_blob(rig: dict, requests: list) -> bytes:
    """The pose blob of sfto_pose_eval / oracle/pose_harness.c."""
    import struct
    out = [b"SFTP", struct.pack("<I", len(rig["bones"]))]
    for bd in rig["bones"]:
        out.append(np.asarray(bd["inverse_bind"], "<f4").tobytes() + np.asarray(bd["local_bind"], "<f4").tobytes())
        out.append(struct.pack("<i", bd["parent"]))
        out.append(np.asarray(bd["base_t"], "<f4").tobytes() + np.asarray(bd["base_r"], "<f4").tobytes() +
                   np.asarray(bd["base_s"], "<f4").tobytes())
    out.append(struct.pack("<I", len(rig["anims"])))
    for an in rig["anims"]:
        out.append(struct.pack("<fII", float(an["duration"]), len(an["samplers"]), len(an["channels"])))
        for ins, outs, step in an["samplers"]:
            out.append(struct.pack("<II", len(ins), step) + np.asarray(ins, "<f4").tobytes() + np.asarray(outs, "<f4").tobytes())
        for smp, node, path in an["channels"]:
            out.append(struct.pack("<iii", smp, node, path))
    out.append(struct.pack("<I", len(requests)))
    for a, t in requests:
        out.append(struct.pack("<if", a, float(t)))
    return b"".join(out)


def oracle_pose(blob: bytes, n_bones: int, n_req: int) -> np.ndarray:
    """[request][posed 0 / global 1][bone][16] from the oracle's restatement."""
    L = lib()
    L.sfto_pose_eval.restype = C.c_int
    L.sfto_pose_eval.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64]
    out = np.zeros(n_req * n_bones * 32, np.float32)
    buf = np.frombuffer(blob, np.uint8)
    rc = L.sfto_pose_eval(buf.ctypes.data_as(C.c_void_p), len(blob), out.ctypes.data_as(C.c_void_p), out.size)
    if rc != n_req:
        raise RuntimeError(f"oracle pose evaluation failed ({rc})")
    return out.reshape(n_req, 2, n_bones, 16)


def reference_pose(blob: bytes, n_bones: int, n_req: int) -> np.ndarray:
    with tempfile.TemporaryDirectory() as td:
        ip, op = os.path.join(td, "p.bin"), os.path.join(td, "o.bin")
        open(ip, "wb").write(blob)
        subprocess.run([os.path.join(REF_DIR, "pose_harness"), ip, op], check=True)
        return np.fromfile(op, np.float32).reshape(n_req, 2, n_bones, 16)


def reference_pose_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "pose_harness"))


def reference_available(samples: int) -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"ref_harness_{samples}x"))


RAY_DTYPE = np.dtype([("T", "<f4", (16,)), ("o", "<f4", (3,)), ("d", "<f4", (3,)), ("max_dist", "<f4"), ("model", "<i4")])
HIT_DTYPE = np.dtype([("hit", "<u4"), ("dist", "<f4"), ("pos", "<f4", (3,)), ("nrm", "<f4", (3,))])


def reference_raycast(blob: bytes, rays: np.ndarray) -> np.ndarray:
    """sft_raycast_instance of the unmodified reference for each ray record (RAY_DTYPE) over the
    scene's models (oracle/ref_harness.c, SFT_RAYCAST mode); HIT_DTYPE records."""
    with tempfile.TemporaryDirectory() as td:
        sp, rp, hp = os.path.join(td, "s.sfts"), os.path.join(td, "r.bin"), os.path.join(td, "h.bin")
        open(sp, "wb").write(blob)
        np.ascontiguousarray(rays, RAY_DTYPE).tofile(rp)
        env = dict(os.environ, SFT_RAYCAST=rp)
        subprocess.run([os.path.join(REF_DIR, "ref_harness_1x"), sp, hp], check=True, stdout=subprocess.DEVNULL, env=env)
        return np.fromfile(hp, HIT_DTYPE)


def reference_dump(blob: bytes, samples: int, frame: int = -1, debug_mode: int = 0) -> list[dict]:
    with tempfile.TemporaryDirectory() as td:
        sp, dp = os.path.join(td, "s.sfts"), os.path.join(td, "r.dump")
        open(sp, "wb").write(blob)
        env = dict(os.environ, SFT_DEBUG_MODE=str(debug_mode))
        subprocess.run([os.path.join(REF_DIR, f"ref_harness_{samples}x"), sp, dp, str(frame)], check=True,
                       stdout=subprocess.DEVNULL, env=env)
        return read_dump(dp)
