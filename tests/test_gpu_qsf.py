"""QSF2 model loading (sft_model_load_qsf, sofren2.c:7816-7967): the atrium_small atrium written
as a QSF2 file (textures, lightmap page, meshlets with flat indices, bounds, cones, the
meshlet-to-mesh table and a prebuilt BLAS) is loaded and drawn through this library's public C
API by a small C program, against the reference's own load and render of the same file
(oracle/qsf_harness.c), frame by frame at 1x and 4x MSAA.  The file's bytes are pinned too, so
both sides are known to read the same file.  Then the reference's own maps (res/simple.qsf and
res/simpleb.qsf, lightmapped, with their own BLAS and game lights), which `make -C oracle ref`
copies beside the reference builds: the viewer's frame loop at 1600x900 (oracle/map_scene.h) and
ray queries against the file's BLAS, against the reference's renders and answers; skipped where
the maps were not copied."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import golden_cases as gc
from sofren2_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_qsf_file_bytes_pinned(golden):
    assert gc.sha(np.frombuffer(gc.qsf_model(), np.uint8)) == golden["qsf"]["file"]


@pytest.fixture(scope="module")
def qsf_exe(gpu_lib):
    out = os.path.join(build.OUT, "qsf_frame")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-std=gnu11", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "qsf_frame.c"), "-o", out, "-L", build.OUT, "-lsofren2_gb300",
                    f"-Wl,-rpath,{build.OUT}", "-lm"], check=True)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("samples", [1, 4])
def test_qsf_model_matches_reference(qsf_exe, golden, samples):
    with tempfile.TemporaryDirectory() as td:
        qp, op = os.path.join(td, "m.qsf"), os.path.join(td, "q.bin")
        with open(qp, "wb") as f:
            f.write(gc.qsf_model())
        r = subprocess.run([qsf_exe, "atrium", qp, op, str(samples)])
        assert r.returncode == 0, f"qsf_frame exited {r.returncode} (5/6/8: a bad or cut file was accepted, 4: the file was rejected)"
        frames = np.fromfile(op, np.uint32).reshape(-1, 360, 640)
    exp = golden["qsf"][str(samples)]
    assert len(frames) == len(exp)
    for k, f in enumerate(frames):
        assert gc.sha(f) == exp[k], f"frame {k} at {samples}x differs from the reference"


@pytest.mark.gpu
@pytest.mark.parametrize("samples", [1, 4])
@pytest.mark.parametrize("name", gc.QSF_MAPS)
def test_reference_map_matches_reference(qsf_exe, golden, name, samples):
    import hashlib
    mp = os.path.join(ROOT, "oracle", "_ref", "res", name + ".qsf")
    if not os.path.exists(mp):
        pytest.skip(f"{name}.qsf was not copied beside the reference builds")
    exp = golden["qsf_maps"][name]
    with open(mp, "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == exp["file"], "a different map file"
    with tempfile.TemporaryDirectory() as td:
        op = os.path.join(td, "m.bin")
        r = subprocess.run([qsf_exe, "map", mp, op, str(samples), "1600", "900"])
        assert r.returncode == 0, f"qsf_frame exited {r.returncode}"
        frames = np.fromfile(op, np.uint32).reshape(-1, 900, 1600)
        rays = np.fromfile(op + ".rays", np.uint32)
    assert len(frames) == len(exp[str(samples)])
    for k, f in enumerate(frames):
        assert gc.sha(f) == exp[str(samples)][k], f"{name} frame {k} at {samples}x differs from the reference"
    assert gc.sha(rays) == exp["rays"], f"{name}: ray queries differ from the reference"
