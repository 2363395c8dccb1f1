"""Readers for the section dumps written by the reference harness and the CPU oracle."""
from __future__ import annotations

import struct
import zlib

import numpy as np

_DT = {"u32": np.uint32, "i32": np.int32, "f32": np.float32, "u64": np.uint64, "u8": np.uint8}


def read_dump(path_or_bytes) -> list[dict]:
    """Returns one dict per frame (keys: section names); model-level sections ('blas') go in frame 0's
    'blas' list."""
    data = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    off, frames, cur, blas = 0, [], {}, []
    while off < len(data):
        assert data[off:off + 4] == b"SEC1", "bad dump section"
        name = data[off + 4:off + 36].split(b"\0")[0].decode()
        dt = data[off + 36:off + 44].split(b"\0")[0].decode()
        (n,) = struct.unpack_from("<Q", data, off + 44)
        body = data[off + 52:off + 52 + n]
        off += 52 + n
        arr = np.frombuffer(body, dtype=_DT[dt]).copy()
        if name == "blas":
            blas.append(arr)
            continue
        if name == "color" and cur:
            frames.append(cur)
            cur = {}
        cur[name] = arr
    if cur:
        frames.append(cur)
    if frames:
        frames[0]["blas"] = blas
    return frames


def tile_lists(frame: dict) -> list[np.ndarray]:
    counts = frame["tile_counts"]
    pays = frame["tile_payloads"]
    out, o = [], 0
    for c in counts:
        out.append(pays[o:o + c])
        o += c
    return out


def write_png(path: str, argb: np.ndarray, w: int, h: int) -> None:
    img = argb.reshape(h, w)
    rgb = np.stack([(img >> 16) & 255, (img >> 8) & 255, img & 255], axis=-1).astype(np.uint8)
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(tag, body):
        return struct.pack(">I", len(body)) + tag + body + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    open(path, "wb").write(png)
