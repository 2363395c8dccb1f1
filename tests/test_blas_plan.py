"""The BLAS shape plan (sofren2_gb300/csrc/sftg_blas_plan.h, the host half of the device
builder) against the node images of the reference's own builds, on the CPU: for every model of
the golden cases and the BLAS edge models, the plan for the model's live-triangle count must give
the reference's node count, leaf flags, slot counts and child indices; each sort level's ranges
must be disjoint and in increasing order."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import golden_cases as gc
from oracle_lib import Oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "sofren2_gb300", "csrc")


@pytest.fixture(scope="module")
def plan_tool(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("plan") / "blas_plan")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", CSRC, os.path.join(ROOT, "tests", "blas_plan.cc"), "-o", exe], check=True)
    return exe


def plans(exe: str, counts: list[int], tmp) -> list[tuple[np.ndarray, list[np.ndarray]]]:
    out = str(tmp / "plans.bin")
    subprocess.run([exe, out] + [str(c) for c in counts], check=True)
    buf = np.fromfile(out, np.uint32)
    res, o = [], 0
    for _ in counts:
        nn, nl = int(buf[o]), int(buf[o + 1]); o += 2
        nodes = buf[o:o + nn * 11].reshape(nn, 11); o += nn * 11
        levels = []
        for _ in range(nl):
            c = int(buf[o]); o += 1
            levels.append(buf[o:o + 2 * c].reshape(c, 2)); o += 2 * c
        res.append((nodes, levels))
    return res


def live_triangles(model) -> int:
    n = 0
    for ms in model.meshes:
        ind = ms.inds.reshape(ms.n, 16, 4, 8)[:, :, :3, :].astype(np.int32)   # [meshlet][batch][v0 v1 v2][lane]
        n += int((~((ind[:, :, 0] == ind[:, :, 1]) & (ind[:, :, 1] == ind[:, :, 2]))).sum())
    return n


@pytest.mark.parametrize("name", gc.BLAS_CASES)
def test_plan_matches_reference_shape(plan_tool, tmp_path, golden, name):
    sc = gc.blas_edge_scene() if name == "blas_edges" else gc.scene(name)
    counts = [live_triangles(m) for m in sc.models]
    o = Oracle(gc.blas_blob(name))
    for mi, ((nodes, levels), n) in enumerate(zip(plans(plan_tool, counts, tmp_path), counts)):
        assert len(nodes) == golden["blas"][name]["nodes"][mi], f"model {mi}: node count"
        ref = np.frombuffer(o.model_blas(mi)[0], np.uint8).reshape(-1, 256)
        child = ref[:, 192:224].copy().view(np.uint32)
        cnt, leaf = ref[:, 224], ref[:, 225]
        for k, (start, count, nchild, *ch) in enumerate(nodes.tolist()):
            if count <= 8:
                assert leaf[k] == 1 and cnt[k] == count, f"model {mi} node {k}: leaf of {count}"
                assert all(c >> 31 for c in child[k, :count]) and all(c == 0xFFFFFFFF for c in child[k, count:])
            else:
                assert leaf[k] == 0 and cnt[k] == nchild, f"model {mi} node {k}: {nchild} children"
                assert child[k].tolist() == ch, f"model {mi} node {k}: child indices"
        for L in levels:
            ends = L[:, 0] + L[:, 1]
            assert (L[:, 1] >= 2).all() and (L[1:, 0] >= ends[:-1]).all() and (ends <= n).all()
