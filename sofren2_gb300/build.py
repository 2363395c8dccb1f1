"""Builds libsofren2_gb300.so (CUDA kernels for sm_103a + the C host runtime) in-tree.

    python -m sofren2_gb300.build            # library only
    python -m sofren2_gb300.build --oracle   # also the CPU oracle (and the reference, when present)

Device code is compiled with -fmad=false: the render path reproduces the reference's
floating-point results bit for bit, so every fused multiply-add is written explicitly.
Host C is compiled with -ffp-contract=off for the same reason.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libsofren2_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["sftg_geom.cu", "sftg_tile.cu", "sftg_occl.cu", "sftg_pose.cu", "sftg_ray.cu", "sftg_blas.cu", "sftg_api.cu"]
C_SOURCES = ["sft_lib.c", "sft_scene.c", "sft_serve.c"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsofren2_gb300")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_library(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, ARCH, "-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-c", s, "-o", o])
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".c", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=gnu11", "-fPIC", "-Wall",
                         "-Wno-unused-function", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"),
                         "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def reference_dir() -> str:
    """Where the reference's sources are read from to (re)build the reference harnesses: the
    directory named by SFT_REFERENCE_DIR, or "" when it is not set.  Harnesses built earlier stay
    in oracle/_ref and keep serving the tests without it."""
    return os.environ.get("SFT_REFERENCE_DIR", "")


def build_oracle_and_reference() -> None:
    """CPU oracle always; the reference harness only where the reference sources exist (x86-64 + AVX2)."""
    oracle_dir = os.path.join(ROOT, "oracle")
    _run(["make", "-s", "-C", oracle_dir, "oracle"])
    ref_dir = reference_dir()
    if ref_dir and os.path.exists(os.path.join(ref_dir, "sofren2.c")) and os.uname().machine == "x86_64":
        _run(["make", "-s", "-C", oracle_dir, "ref", f"REF_DIR={ref_dir}"])
    # the reference's own render path for the timed CPU baseline, native to this host (NEON on
    # aarch64), from the copy of its source that `make ref` left beside the builds
    if os.path.exists(os.path.join(oracle_dir, "_ref", "src", "sofren2.c")):
        try:
            _run(["make", "-s", "-C", oracle_dir, "ref_bench"])
        except RuntimeError as e:   # the baseline then falls back to the oracle port, and says so
            print(f"reference CPU build failed on this host: {str(e).splitlines()[-1][:300]}", file=sys.stderr)


if __name__ == "__main__":
    lib = build_library(force="--force" in sys.argv)
    print(lib)
    if "--oracle" in sys.argv:
        build_oracle_and_reference()
