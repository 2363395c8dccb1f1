"""The load-time builders of include/sofren2.h on the CPU: sft_mesh_build_meshlets (the
reference's greedy meshlet builder with Welzl spheres, normal cones and culling joints,
sofren2.c:2255-2489, 6918-7045, 7467-7660) and sft_model_fit_shadow_proxies (bone-cluster and
BVH-node capsules, sofren2.c:3064-3524), run by tests/model_build.c over the raw models of
tests/raw_models.py (spheres, boxes, a ground grid, the skinned humanoid at two proxy budgets,
a soup of unconnected and degenerate triangles, triangles that repeat a vertex).  Their output
must equal the reference's own builders byte for byte: pinned by digests of
oracle/build_harness.c's output, and compared directly where the reference is compiled here.
The proxies use the BLAS of the oracle's restated builder over the built meshlets, which must
equal the reference's BLAS too."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import golden_cases as gc
import raw_models as rm
from oracle_lib import REF_DIR, Oracle
from sofren2_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAMES = list(rm.models())


@pytest.fixture(scope="module")
def builder(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path_factory.mktemp("mb") / "model_build")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=gnu11", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "model_build.c"), os.path.join(ROOT, "tests", "sftg_fake.c"), "-o", exe, "-lm"],
                   check=True)
    return exe


def _build(exe, name, td, blas=None):
    ip, op = os.path.join(td, name + ".bin"), os.path.join(td, name + ".out")
    with open(ip, "wb") as f:
        f.write(rm.blob(name))
    args = [exe, ip, op]
    if blas is not None:
        bp = os.path.join(td, name + ".blas")
        with open(bp, "wb") as f:
            f.write(blas[0])
        args += [bp, str(blas[1])]
    subprocess.run(args, check=True)
    return rm.read_output(op, name, False)


def _oracle_blas(out, name):
    sc = scenes.Scene()
    sc.add_model(rm.as_scene_model(out, name))
    o = Oracle(sc.to_bytes())
    try:
        return o.model_blas(0)
    finally:
        o.close()


@pytest.mark.parametrize("name", NAMES)
def test_meshlets_blas_proxies_match_reference_digests(builder, golden, name, tmp_path):
    g = golden["model_build"][name]
    out = _build(builder, name, str(tmp_path))
    assert [d["n"] for d in out["meshes"]] == g["meshlets"]
    assert gc.sha(np.frombuffer(rm.meshlet_bytes(out), np.uint8)) == g["meshlet_sha256"], f"{name}: meshlets differ from the reference's"
    blas, root = _oracle_blas(out, name)
    assert (len(blas) // 256, root) == (g["blas_nodes"], g["blas_root"])
    assert gc.sha(np.frombuffer(blas, np.uint8)) == g["blas_sha256"]
    out2 = _build(builder, name, str(tmp_path), (blas, root))
    assert out2["proxies"].shape[0] == g["proxies"]
    assert gc.sha(out2["proxies"]) == g["proxy_sha256"], f"{name}: shadow proxies differ from the reference's"


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_DIR, "build_harness")), reason="reference not compiled here (oracle/_ref)")
@pytest.mark.parametrize("name", ["humanoid", "soup"])
def test_builders_equal_reference_with_other_seed(builder, name, tmp_path):
    """Another rand() seed: different Welzl draws, still the reference's bytes."""
    seed, budget, bones, meshes = rm.models()[name]
    import struct
    raw = bytearray(rm.blob(name))
    raw[8:12] = struct.pack("<I", seed + 1000)
    ip = str(tmp_path / "in.bin")
    with open(ip, "wb") as f:
        f.write(bytes(raw))
    subprocess.run([os.path.join(REF_DIR, "build_harness"), ip, str(tmp_path / "ref.out")], check=True)
    ref = rm.read_output(str(tmp_path / "ref.out"), name, True)
    bp = str(tmp_path / "b.blas")
    with open(bp, "wb") as f:
        f.write(ref["blas"])
    subprocess.run([builder, ip, str(tmp_path / "ours.out"), bp, str(ref["blas_root"])], check=True)
    ours = rm.read_output(str(tmp_path / "ours.out"), name, False)
    assert rm.meshlet_bytes(ours) == rm.meshlet_bytes(ref)
    assert np.array_equal(ours["proxies"], ref["proxies"])


def test_meshlet_builder_rejects_out_of_range_indices(builder, tmp_path):
    """A triangle naming a vertex past the end: no meshlets, no read outside the arrays."""
    import struct
    m = scenes.uv_sphere(8, 4, 0.5)
    bad = m.tris.copy()
    bad[2, 1] = len(m.pos)
    raw = [b"SFTR", struct.pack("<IIiI", 1, 1, 0, 0), struct.pack("<I", 1),
           struct.pack("<III", len(m.pos), len(bad), 0), m.pos.astype("<f4").tobytes(), m.nrm.astype("<f4").tobytes(),
           m.uv.astype("<f4").tobytes(), bad.astype("<i4").tobytes()]
    ip, op = str(tmp_path / "bad.bin"), str(tmp_path / "bad.out")
    with open(ip, "wb") as f:
        f.write(b"".join(raw))
    subprocess.run([builder, ip, op], check=True)
    assert np.fromfile(op, np.uint32)[0] == 0
