"""The device emulation of the x86 approximations (sofren2_gb300/csrc/sftg_lane.cuh) on the GPU,
for all 2^32 input bit patterns: RCPPS and RSQRTPS through their fast paths equal the plain table
form (tests/lane_check.cu, compiled here for sm_103a)."""
import os
import shutil
import subprocess

import pytest

from sofren2_gb300 import build

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_rcp_rsqrt_fast_paths_exhaustive(tmp_path, gpu_lib):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "lane_check")
    subprocess.run([nvcc, build.ARCH, "-O3", "-fmad=false", "-std=c++17", "-I", os.path.join(ROOT, "sofren2_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "lane_check.cu"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    rcp_bad, rsq_bad, first_rcp, first_rsq = r.stdout.split()
    assert r.returncode == 0 and rcp_bad == "0" and rsq_bad == "0", r.stdout
