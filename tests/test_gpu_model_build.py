"""sft_model_build on the GPU path: the ground, shapes and humanoid raw models
(tests/raw_models.py) built by this library (meshlets and shadow proxies on the host, the BLAS on
the device) and rendered through the public C API by tests/model_build_frame.c, frame for frame
equal to the reference building the same models with its own builders and rendering the same
calls (oracle/build_harness.c, oracle/build_scene.h), at 1x and 4x MSAA: capsule shadows of the
fitted proxies and the occlusion through the device-built BLAS included."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import golden_cases as gc
import raw_models as rm
from sofren2_gb300 import build

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def frame_exe(gpu_lib):
    out = os.path.join(build.OUT, "model_build_frame")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-std=gnu11", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "model_build_frame.c"), "-o", out, "-L", build.OUT, "-lsofren2_gb300",
                    f"-Wl,-rpath,{build.OUT}", "-lm"], check=True)
    return out


@pytest.mark.parametrize("samples", [1, 4])
def test_built_models_render_like_reference(frame_exe, golden, samples):
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for n in ("ground", "shapes", "humanoid"):
            p = os.path.join(td, n + ".bin")
            with open(p, "wb") as f:
                f.write(rm.blob(n))
            paths.append(p)
        op = os.path.join(td, "frames.bin")
        r = subprocess.run([frame_exe, op, str(samples)] + paths)
        assert r.returncode == 0, f"model_build_frame exited {r.returncode}"
        frames = np.fromfile(op, np.uint32).reshape(-1, 360, 640)
    exp = golden["model_build"]["frames"][str(samples)]
    assert len(frames) == len(exp)
    for k, f in enumerate(frames):
        assert gc.sha(f) == exp[k], f"frame {k} at {samples}x differs from the reference's render of its own build"
