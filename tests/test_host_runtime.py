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


def _load_qsf(host, path):
    host.sft_model_load_qsf.restype = C.c_void_p
    host.sft_model_load_qsf.argtypes = [C.c_char_p, C.c_void_p]
    host.sft_model_get_meshlet_count.restype = C.c_uint32
    host.sft_model_get_meshlet_count.argtypes = [C.c_void_p]
    host.sft_model_get_blas.restype = C.c_void_p
    host.sft_model_get_blas.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    m = host.sft_model_load_qsf(path.encode(), None)
    if not m:
        return None
    n, root = C.c_uint32(0), C.c_uint32(0)
    host.sft_model_get_blas(m, C.byref(n), C.byref(root))
    return int(host.sft_model_get_meshlet_count(m)), int(n.value), int(root.value)


def test_qsf_loader_on_the_host(host, golden, tmp_path):
    """sft_model_load_qsf (sofren2.c:7816-7967) parses a QSF2 file on the host: the atrium file the
    tests write, with its BLAS, and the reference's own maps (53 and 84 meshlets, 585 BLAS nodes)
    where they are built here."""
    data = gc.qsf_model()
    p = tmp_path / "atrium.qsf"
    p.write_bytes(data)
    sc = gc.scene("atrium_small")
    got = _load_qsf(host, str(p))
    assert got == (sum(ms.n for ms in sc.models[0].meshes), golden["blas"]["atrium_small"]["nodes"][0], 0)
    res = os.path.join(ROOT, "oracle", "_ref", "res")
    for name, meshlets in (("simple", 53), ("simpleb", 84)):
        f = os.path.join(res, name + ".qsf")
        if os.path.exists(f):
            assert _load_qsf(host, f) == (meshlets, 585, _load_qsf(host, f)[2])


def test_qsf_loader_rejects_broken_files(host, tmp_path):
    """Truncated files (cut inside the header, the textures, the meshlets or the BLAS), a wrong
    magic and a wrong version are refused with NULL, never read past their end."""
    data = gc.qsf_model()
    cuts = [0, 3, 8, 16, 20, 200, len(data) // 4, len(data) // 2, len(data) - 256 * 3, len(data) - 1]
    for cut in cuts:
        p = tmp_path / f"cut{cut}.qsf"
        p.write_bytes(data[:cut])
        assert _load_qsf(host, str(p)) is None, f"a file cut at {cut} of {len(data)} bytes was accepted"
    bad = bytearray(data); bad[0:4] = b"QSF1"
    (tmp_path / "magic.qsf").write_bytes(bytes(bad))
    assert _load_qsf(host, str(tmp_path / "magic.qsf")) is None
    bad = bytearray(data); bad[4:8] = (3).to_bytes(4, "little")
    (tmp_path / "version.qsf").write_bytes(bytes(bad))
    assert _load_qsf(host, str(tmp_path / "version.qsf")) is None
    assert _load_qsf(host, str(tmp_path / "missing.qsf")) is None
