"""Regenerates tests/golden/golden.json from the reference itself.

Requires the reference sources (sofren2_gb300.build.reference_dir(): SFT_REFERENCE_DIR) on an x86-64 host
with AVX2: `make -C oracle ref` compiles them unmodified into oracle/_ref, and each golden case
(tests/golden_cases.py) is rendered by that binary with one worker thread.  Stored per case and
sample count: the SHA-256 of the scene blob and of every dump section, the live meshlet list
and the number of used clip slots, plus the reference's sft_present time.

    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
sys.path.insert(0, TESTS)
sys.path.insert(0, ROOT)

import golden_cases as gc  # noqa: E402
from oracle_lib import reference_dump  # noqa: E402


def main(names: list[str]) -> None:
    from sofren2_gb300.build import reference_dir
    ref_dir = reference_dir()
    if not ref_dir:
        raise SystemExit("set SFT_REFERENCE_DIR to the reference project's checkout")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF_DIR={ref_dir}"], check=True)
    path = os.path.join(HERE, "golden.json")
    golden = json.load(open(path)) if os.path.exists(path) else {}
    for name in [n for n in names if n in gc.CASES] if names else list(gc.CASES):
        blob = gc.blob(name)
        entry = {"generator": gc.CASES[name][0], "kwargs": gc.CASES[name][1], "scene_sha256": gc.sha(memoryview(blob)),
                 "samples": {}}
        for S in gc.SAMPLES[name]:
            frame = reference_dump(blob, S)[0]
            d, live = gc.digests(frame, lights=gc.n_lights(name))
            d["live_meshlets"] = live
            d["reference_present_ms"] = float(frame["present_ns"][0]) / 1e6
            entry["samples"][str(S)] = d
            print(name, S, "payloads", int(frame["tile_counts"].sum()), "clips", d["clip_used"], flush=True)
        golden[name] = entry
    if not names or "debug" in names:
        # colour digests of the debug views (sft_set_debug_mode through SFT_DEBUG_MODE)
        dbg = {}
        for name, mode, S in gc.DEBUG_CASES:
            frame = reference_dump(gc.blob(name), S, debug_mode=mode)[0]
            dbg[f"{name}/{mode}/{S}"] = gc.sha(frame["color"])
            print("debug", name, mode, S, flush=True)
        golden["debug_views"] = dbg
    if not names or "blas" in names:
        # every model's BLAS node images as the reference builds them (the harness's blas
        # sections), for the golden cases and the BLAS edge models
        bl = {}
        for name in gc.BLAS_CASES:
            frame = reference_dump(gc.blas_blob(name), 1, frame=0)[0]
            bl[name] = {"nodes": [len(b) // 256 for b in frame["blas"]], "sha256": [gc.sha(b) for b in frame["blas"]]}
            print("blas", name, bl[name]["nodes"], flush=True)
        golden["blas"] = bl
    if not names or "tlas" in names:
        # frame 0's TLAS as the reference's host code builds it (padding bytes left out, as the
        # reference leaves them unset)
        from compare import _nodes_meaningful
        tl = {}
        for name in gc.CASES:
            raw = reference_dump(gc.blob(name), 1, frame=0)[0].get("tlas")
            nodes = _nodes_meaningful(raw) if raw is not None else None
            tl[name] = {"nodes": 0 if nodes is None else int(nodes.shape[0]), "sha256": gc.sha(nodes if nodes is not None else b"")}
            print("tlas", name, tl[name]["nodes"], flush=True)
        golden["tlas"] = tl
    if not names or "pose" in names:
        # sft_pose_update of the reference on a seeded rig (oracle/pose_harness.c)
        from oracle_lib import pose_blob, reference_pose
        from sofren2_gb300 import scenes
        rig = scenes.pose_rig()
        req = scenes.pose_requests(rig, 60)
        out = reference_pose(pose_blob(rig, req), len(rig["bones"]), len(req))
        golden["pose"] = {"rig_seed": 6001, "requests": len(req), "sha256": gc.sha(out)}
        print("pose", golden["pose"]["sha256"][:16], flush=True)
    if not names or "soa_math" in names:
        # the reference's SoA math helpers (oracle/soa_harness.c) on tests/test_soa_math.soa_inputs()
        import tempfile
        import numpy as np
        from test_soa_math import soa_inputs
        with tempfile.TemporaryDirectory() as td:
            ip, op = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
            soa_inputs().tofile(ip)
            subprocess.run([os.path.join(ROOT, "oracle", "_ref", "soa_harness"), ip, op], check=True)
            golden["soa_math"] = {"seed": 7001, "groups": 512, "sha256": gc.sha(np.fromfile(op, np.uint32))}
        print("soa_math", golden["soa_math"]["sha256"][:16], flush=True)
    if not names or "model_build" in names:
        # the reference's load-time builders on raw meshes (oracle/build_harness.c): meshlets, BLAS and
        # proxies per model of tests/raw_models.py, and its renders of oracle/build_scene.h over them
        import tempfile
        import numpy as np
        import raw_models as rm
        mb = {}
        with tempfile.TemporaryDirectory() as td:
            for n in rm.models():
                ip, op = os.path.join(td, n + ".bin"), os.path.join(td, n + ".out")
                open(ip, "wb").write(rm.blob(n))
                subprocess.run([os.path.join(ROOT, "oracle", "_ref", "build_harness"), ip, op], check=True)
                out = rm.read_output(op, n, True)
                mb[n] = {"meshlets": [int(d["n"]) for d in out["meshes"]], "meshlet_sha256": gc.sha(np.frombuffer(rm.meshlet_bytes(out), np.uint8)),
                         "proxies": int(out["proxies"].shape[0]), "proxy_sha256": gc.sha(out["proxies"]),
                         "blas_nodes": len(out["blas"]) // 256, "blas_root": out["blas_root"],
                         "blas_sha256": gc.sha(np.frombuffer(out["blas"], np.uint8))}
                print("model_build", n, mb[n]["meshlets"], mb[n]["proxies"], flush=True)
            frames = {}
            for S, exe in ((1, "build_harness"), (4, "build_harness_4x")):
                fp = os.path.join(td, f"frames{S}.bin")
                subprocess.run([os.path.join(ROOT, "oracle", "_ref", exe), "render", fp] +
                               [os.path.join(td, n + ".bin") for n in ("ground", "shapes", "humanoid")], check=True)
                frames[str(S)] = [gc.sha(f) for f in np.fromfile(fp, np.uint32).reshape(-1, 360, 640)]
            mb["frames"] = frames
        golden["model_build"] = mb
    if not names or "dmesh" in names:
        # the dynamic-mesh scene (oracle/dmesh_scene.h) rendered by the reference, per frame
        import tempfile
        import numpy as np
        dm = {}
        for S in (1, 4):
            with tempfile.TemporaryDirectory() as td:
                op = os.path.join(td, "dm.bin")
                subprocess.run([os.path.join(ROOT, "oracle", "_ref", f"dmesh_harness_{S}x"), op], check=True)
                frames = np.fromfile(op, np.uint32).reshape(-1, 360, 640)
                dm[str(S)] = [gc.sha(f) for f in frames]
        golden["dmesh"] = dm
        print("dmesh", {k: [h[:12] for h in v] for k, v in dm.items()}, flush=True)
    if not names or "qsf" in names:
        # the QSF scene (oracle/qsf_scene.h) over the atrium_small atrium written as a QSF2 file,
        # loaded and rendered by the reference, per frame
        import tempfile
        import numpy as np
        data = gc.qsf_model()
        q = {"file": gc.sha(np.frombuffer(data, np.uint8))}
        for S in (1, 4):
            with tempfile.TemporaryDirectory() as td:
                qp, op = os.path.join(td, "m.qsf"), os.path.join(td, "q.bin")
                open(qp, "wb").write(data)
                subprocess.run([os.path.join(ROOT, "oracle", "_ref", f"qsf_harness_{S}x"), "atrium", qp, op], check=True)
                frames = np.fromfile(op, np.uint32).reshape(-1, 360, 640)
                q[str(S)] = [gc.sha(f) for f in frames]
        golden["qsf"] = q
        print("qsf", {k: (v[:12] if isinstance(v, str) else [h[:12] for h in v]) for k, v in q.items()}, flush=True)
    if not names or "maps" in names:
        # the viewer's frame loop (oracle/map_scene.h) over the reference's own QSF2 maps at 1600x900,
        # per frame, and its ray queries; `make ref` copies the maps to oracle/_ref/res
        import hashlib
        import tempfile
        import numpy as np
        maps = {}
        for m in gc.QSF_MAPS:
            mp = os.path.join(ROOT, "oracle", "_ref", "res", m + ".qsf")
            e = {"file": hashlib.sha256(open(mp, "rb").read()).hexdigest()}
            for S in (1, 4):
                with tempfile.TemporaryDirectory() as td:
                    op = os.path.join(td, "m.bin")
                    subprocess.run([os.path.join(ROOT, "oracle", "_ref", f"qsf_harness_{S}x"), "map", mp, op, "1600", "900"], check=True)
                    frames = np.fromfile(op, np.uint32).reshape(-1, 900, 1600)
                    e[str(S)] = [gc.sha(f) for f in frames]
                    rays = np.fromfile(op + ".rays", np.uint32)
                    if S == 1:
                        e["rays"] = gc.sha(rays)
                    assert gc.sha(rays) == e["rays"], "ray queries depend on the MSAA build"
            maps[m] = e
        golden["qsf_maps"] = maps
        print("qsf_maps", {k: [h[:10] for h in v["1"]] for k, v in maps.items()}, flush=True)
    if not names or "raycast" in names:
        # sft_raycast_instance of the reference over seeded rays per case (golden_cases.rays)
        from oracle_lib import reference_raycast
        rc = {}
        for n in gc.RAY_CASES:
            r = gc.rays(n)
            hits = reference_raycast(gc.blob(n), r)
            rc[n] = {"rays": gc.sha(r), "hits": gc.sha(hits), "n_hit": int(hits["hit"].sum())}
        golden["raycast"] = rc
        print("raycast", {k: (v["hits"][:12], v["n_hit"]) for k, v in rc.items()}, flush=True)
    json.dump(golden, open(path, "w"), indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1:])
