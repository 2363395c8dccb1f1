"""The host runtime (include/sofren2.h through sofren2_gb300/csrc/sft_lib.c, and the scene player
sft_scene.c, both compiled unchanged) on the CPU, over a fake of the GPU ABI (tests/sftg_fake.c):
each golden case's frame 0 goes through the public API (scene load, lights, camera, instances,
sft_present), and the TLAS the runtime builds on the host (sft__tlas_build, sofren2.c:3619-3703,
from each model's bounds) must equal the reference's own TLAS for that frame, node for node."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import golden_cases as gc
from compare import _nodes_meaningful

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "sofren2_gb300", "csrc")


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    so = str(tmp_path_factory.mktemp("host") / "libhostfake.so")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=gnu11", "-fPIC", "-shared", "-I",
                    os.path.join(ROOT, "include"), "-I", CSRC, os.path.join(CSRC, "sft_lib.c"), os.path.join(CSRC, "sft_scene.c"),
                    os.path.join(ROOT, "tests", "sftg_fake.c"), "-o", so, "-lm", "-lpthread"], check=True)
    L = C.CDLL(so)
    L.sft_init.argtypes = [C.c_int32, C.c_int32, C.c_int32]
    L.sftx_scene_load.restype, L.sftx_scene_load.argtypes = C.c_void_p, [C.c_void_p, C.c_uint64]
    L.sftx_scene_render.restype = C.c_int
    L.sftx_scene_render.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_int32]
    L.sftx_scene_free.argtypes = [C.c_void_p]
    L.fk_tlas.restype = C.c_uint32
    L.fk_tlas.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    L.sft_init(640, 360, 1)
    return L


@pytest.mark.parametrize("name", list(gc.CASES))
def test_host_tlas_matches_reference(host, golden, name):
    sc = gc.scene(name)
    blob = gc.blob(name)
    buf = np.frombuffer(blob, np.uint8)
    h = host.sftx_scene_load(buf.ctypes.data, len(blob))
    assert h, "scene rejected"
    try:
        f = sc.frames[0]
        color = np.zeros(f.width * f.height, np.uint32)
        assert host.sftx_scene_render(h, 0, color.ctypes.data, 0) == 0
        root, frames = C.c_uint32(0), C.c_uint32(0)
        n = host.fk_tlas(None, 0, C.byref(root), C.byref(frames))
        nodes = np.zeros(max(1, n) * 256, np.uint8)
        host.fk_tlas(nodes.ctypes.data, n, None, None)
    finally:
        host.sftx_scene_free(h)
    exp = golden["tlas"][name]
    assert n == exp["nodes"], f"{n} TLAS nodes, reference {exp['nodes']}"
    got = _nodes_meaningful(nodes[: n * 256]) if n else b""
    assert gc.sha(got) == exp["sha256"], "the host TLAS differs from the reference's"
    assert root.value == 0
