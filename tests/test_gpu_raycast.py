"""Ray queries (sft_raycast_instance, sofren2.c:3733-3837): seeded rays per case (aimed at the
models, random and axis-aligned directions, scaled instance transforms, short distance limits,
zero directions) answered by the oracle and by the GPU through sft_raycast_batch, against the
reference's own answers for the same rays, record for record; a larger set against the oracle;
and the soft cases of the API (no instance, no model)."""
import ctypes as C

import numpy as np
import pytest

import golden_cases as gc
from oracle_lib import Oracle


@pytest.mark.parametrize("name", gc.RAY_CASES)
def test_oracle_raycast_matches_reference(golden, name):
    r = gc.rays(name)
    assert gc.sha(r) == golden["raycast"][name]["rays"], "ray generator changed"
    hits = Oracle(gc.blob(name)).raycast(r)
    assert int(hits["hit"].sum()) == golden["raycast"][name]["n_hit"]
    assert gc.sha(hits) == golden["raycast"][name]["hits"]


@pytest.fixture(scope="module")
def ray_scenes(renderer):
    hs = {n: renderer.load_scene(gc.blob(n)) for n in gc.RAY_CASES}
    yield hs
    for h in hs.values():
        renderer.free_scene(h)


@pytest.mark.gpu
@pytest.mark.parametrize("name", gc.RAY_CASES)
def test_gpu_raycast_matches_reference(renderer, ray_scenes, golden, name):
    r = gc.rays(name)
    hits = renderer.raycast(ray_scenes[name], r)
    if gc.sha(hits) != golden["raycast"][name]["hits"]:
        exp = Oracle(gc.blob(name)).raycast(r)
        diff = [k for k in range(len(r)) if hits[k].tobytes() != exp[k].tobytes()]
        pytest.fail(f"{len(diff)} of {len(r)} rays differ from the reference; first {diff[:5]}: {hits[diff[:2]]} vs {exp[diff[:2]]}")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["atrium_small", "variety"])
def test_gpu_raycast_large_set_matches_oracle(renderer, ray_scenes, name):
    r = gc.rays(name, n=1 << 15, seed=77)
    got = renderer.raycast(ray_scenes[name], r)
    exp = Oracle(gc.blob(name)).raycast(r)
    assert got.tobytes() == exp.tobytes()


@pytest.mark.gpu
def test_gpu_raycast_soft_cases(renderer, ray_scenes):
    from sofren2_gb300.runtime import SftInstance, SftRayHit
    lib = renderer.lib
    v3 = C.c_float * 3
    for inst in (None, SftInstance()):   # no instance; an instance without a model
        ptrs = (C.c_void_p * 1)(C.addressof(inst) if inst is not None else None)
        o, d, md = v3(0, 0, 0), v3(0, 0, 1), (C.c_float * 1)(7.5)
        out = (SftRayHit * 1)()
        out[0].hit = 9
        lib.sft_raycast_batch(ptrs, o, d, md, 1, out)
        assert out[0].hit == 0 and out[0].distance == np.float32(7.5)
