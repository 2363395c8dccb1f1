"""Section-by-section comparison of render dumps (reference harness, CPU oracle, GPU library)."""
from __future__ import annotations

import numpy as np

from oracle_io import tile_lists

NODE_FIELDS = 6 * 8 * 4 + 8 * 4 + 2   # SoA AABBs, child indices, child_count, is_leaf_group


def _nodes_meaningful(raw: np.ndarray) -> np.ndarray:
    """Strips the padding bytes of sft_bvh_node images (256 B each), which the reference leaves unset."""
    n = raw.size // 256
    return raw[: n * 256].reshape(n, 256)[:, :NODE_FIELDS]


def compare_frames(ref: dict, other: dict, samples: int, n_lights: int = 64) -> dict:
    """Returns {section: mismatch count} (0 everywhere means bit-exact).  light_vis is compared
    for the frame's first min(n_lights, 64) lights: the reference writes no other column
    (sofren2.c:8166-8173)."""
    out = {}
    out["color"] = int(np.count_nonzero(ref["color"] != other["color"]))
    out["color_max_lsb"] = int(np.max(np.abs(
        np.stack([(ref["color"] >> s) & 255 for s in (16, 8, 0)]).astype(np.int32)
        - np.stack([(other["color"] >> s) & 255 for s in (16, 8, 0)]).astype(np.int32)))) if ref["color"].size else 0
    out["tile_counts"] = int(np.count_nonzero(ref["tile_counts"] != other["tile_counts"]))
    if out["tile_counts"] == 0:
        out["tile_payloads"] = int(np.count_nonzero(ref["tile_payloads"] != other["tile_payloads"]))
    else:
        out["tile_payloads"] = -1
    out["vid"] = int(np.count_nonzero(ref["vid"] != other["vid"]))
    out["depth"] = int(np.count_nonzero(ref["depth"].view(np.uint32) != other["depth"].view(np.uint32)))
    rs, os_ = ref["ss_cache"].view(np.uint32), other["ss_cache"].view(np.uint32)
    if rs.size == os_.size:
        live = rs.reshape(-1, 9 * 64)
        mask = ~np.all(live == 0xFFFFFFFF, axis=1)
        out["ss_cache"] = int(np.count_nonzero(live[mask] != os_.reshape(-1, 9 * 64)[mask]))
    else:
        out["ss_cache"] = -1
    # the reference reserves clip slots 64 at a time (sofren2.c:4356-4361): only its used prefix compares
    rc, oc = ref["clip"].view(np.uint32), other["clip"].view(np.uint32)
    n = min(rc.size, oc.size)
    out["clip"] = int(np.count_nonzero(rc[:n] != oc[:n])) if (rc.size == oc.size or rc.size % (64 * 41) == 0) else -1
    nl = min(n_lights, 64)
    out["light_vis"] = int(np.count_nonzero(ref["light_vis"].reshape(-1, 64)[:, :nl] != other["light_vis"].reshape(-1, 64)[:, :nl])) \
        if ref["light_vis"].size == other["light_vis"].size else -1
    if "tlas" in ref and "tlas" in other:
        a, b = _nodes_meaningful(ref["tlas"]), _nodes_meaningful(other["tlas"])
        out["tlas"] = int(np.count_nonzero(a != b)) if a.shape == b.shape else -1
    return out


def first_vid_mismatch(ref: dict, other: dict, cols: int, samples: int):
    per = 4096 * samples
    d = np.nonzero(ref["vid"] != other["vid"])[0]
    if not d.size:
        return None
    i = int(d[0])
    tile, r = divmod(i, per)
    s, p = divmod(r, 4096)
    y, x = divmod(p, 64)
    return dict(tile=tile, sample=s, x=(tile % cols) * 64 + x, y=(tile // cols) * 64 + y,
                ref=hex(int(ref["vid"][i])), other=hex(int(other["vid"][i])),
                ref_depth=float(ref["depth"][i]), other_depth=float(other["depth"][i]))
