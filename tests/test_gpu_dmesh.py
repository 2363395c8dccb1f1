"""Dynamic meshes (sft_dmesh_*, sft_draw_cube / _cube_inv / _sphere / _capsule / _cylinder,
quads with four normals, triangles, alloc_quads batches, a mesh pushed past its capacity)
drawn through this library's public C API by a small C program, against the reference's own
renders of the same calls (oracle/dmesh_harness.c), frame by frame at 1x and 4x MSAA."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import golden_cases as gc
from sofren2_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def dmesh_exe(gpu_lib):
    out = os.path.join(build.OUT, "dmesh_frame")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-std=gnu11", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "dmesh_frame.c"), "-o", out, "-L", build.OUT, "-lsofren2_gb300",
                    f"-Wl,-rpath,{build.OUT}", "-lm"], check=True)
    return out


@pytest.mark.parametrize("samples", [1, 4])
def test_dmesh_scene_matches_reference(dmesh_exe, golden, samples):
    with tempfile.TemporaryDirectory() as td:
        op = os.path.join(td, "dm.bin")
        subprocess.run([dmesh_exe, op, str(samples)], check=True)
        frames = np.fromfile(op, np.uint32).reshape(-1, 360, 640)
    exp = golden["dmesh"][str(samples)]
    assert len(frames) == len(exp)
    for k, f in enumerate(frames):
        assert gc.sha(f) == exp[k], f"frame {k} at {samples}x differs from the reference"
