"""BLAS construction (sft__blas_build_model, sofren2.c:3526-3617, over the 8-wide builder
2895-3062): every model of the golden cases and of the BLAS edge models (one leaf, one split,
all centroids equal, a flat lattice, padding between meshes, 60000 triangles on a grid, a single
triangle, only padding), as node images byte for byte against the reference's own build.  The oracle is pinned on the CPU;
the device build (at model creation) is read back through sft_model_get_blas."""
import numpy as np
import pytest

import golden_cases as gc
from oracle_lib import Oracle


@pytest.mark.parametrize("name", gc.BLAS_CASES)
def test_oracle_blas_matches_reference(golden, name):
    exp = golden["blas"][name]
    o = Oracle(gc.blas_blob(name))
    for mi, (n, digest) in enumerate(zip(exp["nodes"], exp["sha256"])):
        nodes, root = o.model_blas(mi)
        assert len(nodes) // 256 == n, f"model {mi}: {len(nodes) // 256} nodes, reference {n}"
        assert root == 0
        assert gc.sha(np.frombuffer(nodes, np.uint8)) == digest, f"model {mi} differs from the reference's BLAS"


@pytest.mark.gpu
@pytest.mark.parametrize("name", gc.BLAS_CASES)
def test_gpu_blas_matches_reference(renderer, golden, name):
    exp = golden["blas"][name]
    h = renderer.load_scene(gc.blas_blob(name))
    try:
        for mi, (n, digest) in enumerate(zip(exp["nodes"], exp["sha256"])):
            nodes, root = renderer.model_blas(h, mi)
            assert len(nodes) // 256 == n, f"model {mi}: {len(nodes) // 256} nodes, reference {n}"
            assert root == 0
            if gc.sha(np.frombuffer(nodes, np.uint8)) != digest:
                ref, _ = Oracle(gc.blas_blob(name)).model_blas(mi)
                bad = [k for k in range(n) if nodes[k * 256:(k + 1) * 256] != ref[k * 256:(k + 1) * 256]]
                pytest.fail(f"model {mi}: {len(bad)} of {n} nodes differ from the reference's BLAS; first {bad[:5]}")
    finally:
        renderer.free_scene(h)
