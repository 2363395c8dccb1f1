"""Skeletal poses on the GPU (sftg_pose_eval, one warp per request) against the oracle's
restatement of sft_pose_update, which matches the reference bit for bit.  The device's acosf,
sinf and cosf round differently from the host libm inside the quaternion slerp, so matrices are
compared with a tolerance of 2e-5 relative to each matrix's largest entry."""
import numpy as np
import pytest

from oracle_lib import oracle_pose, pose_blob
from sofren2_gb300 import scenes

pytestmark = pytest.mark.gpu

TOL = 2e-5


@pytest.mark.parametrize("seed", [6001, 6002, 6003])
def test_pose_eval_matches_oracle(renderer, seed):
    rig = scenes.pose_rig(seed)
    nb = len(rig["bones"])
    req = scenes.pose_requests(rig, 90, seed=seed)
    ref = oracle_pose(pose_blob(rig, req), nb, len(req))
    sk = renderer.skeleton_upload(rig)
    posed, glob = renderer.pose_eval([(sk, a, t) for a, t in req], [nb] * len(req))
    posed = posed.reshape(len(req), nb, 16)
    glob = glob.reshape(len(req), nb, 16)
    for k, (a, _) in enumerate(req):
        if a < 0 or a >= len(rig["anims"]):
            assert not posed[k].any(), "an out-of-range animation must leave the matrices untouched"
            continue
        for got, exp in ((posed[k], ref[k, 0]), (glob[k], ref[k, 1])):
            scale = np.abs(exp).max(axis=1, keepdims=True) + 1e-6
            err = (np.abs(got - exp) / scale).max()
            assert err <= TOL, f"request {k}: relative error {err:.2e}"


def test_pose_eval_batches_several_skeletons(renderer):
    rigs = [scenes.pose_rig(7001, n_bones=9), scenes.pose_rig(7002, n_bones=40)]
    ids = [renderer.skeleton_upload(r) for r in rigs]
    reqs, counts, refs = [], [], []
    for sk, rig in zip(ids, rigs):
        rq = scenes.pose_requests(rig, 12, seed=sk)
        refs.append(oracle_pose(pose_blob(rig, rq), len(rig["bones"]), len(rq)))
        reqs += [(sk, a, t) for a, t in rq]
        counts += [len(rig["bones"])] * len(rq)
    posed, _ = renderer.pose_eval(reqs, counts)
    off = 0
    for r, rig in zip(refs, rigs):
        nb = len(rig["bones"])
        for k in range(r.shape[0]):
            got = posed[off * 16:(off + nb) * 16].reshape(nb, 16)
            exp = r[k, 0]
            if exp.any():
                assert (np.abs(got - exp) / (np.abs(exp).max(axis=1, keepdims=True) + 1e-6)).max() <= TOL
            off += nb


def test_sft_pose_update_through_the_api(renderer):
    """sft_model_set_skeleton + sft_pose_create + sft_pose_update on a scene's skinned model give
    the matrices sftg_pose_eval computes for the same rig and time."""
    import ctypes as C

    import golden_cases as gc
    from sofren2_gb300 import runtime

    L = renderer.lib
    L.sftx_scene_model.restype, L.sftx_scene_model.argtypes = C.c_void_p, [C.c_void_p, C.c_uint32]
    L.sft_model_set_skeleton.restype = C.c_int32
    L.sft_model_set_skeleton.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]
    L.sft_pose_create.restype, L.sft_pose_create.argtypes = C.c_void_p, [C.c_void_p, C.c_void_p]
    L.sft_pose_update.restype, L.sft_pose_update.argtypes = None, [C.c_void_p, C.c_int32, C.c_float]
    sc = gc.scene("skinned_small")
    mi = next(i for i, m in enumerate(sc.models) if m.bone_count > 0)
    nb = sc.models[mi].bone_count
    h = renderer.load_scene(gc.blob("skinned_small"))
    try:
        model = L.sftx_scene_model(h, mi)
        rig = scenes.pose_rig(6101, n_bones=nb)
        # the same rig through the C ABI, for the expected matrices
        sk = renderer.skeleton_upload(rig)
        exp, exp_g = renderer.pose_eval([(sk, 0, 0.37)], [nb])
        # and through the public API
        bones = (runtime.SftgBoneDesc * nb)()
        for i, bd in enumerate(rig["bones"]):
            bones[i].inverse_bind[:] = [float(x) for x in np.asarray(bd["inverse_bind"]).reshape(-1)]
            bones[i].local_bind[:] = [float(x) for x in np.asarray(bd["local_bind"]).reshape(-1)]
            bones[i].parent = bd["parent"]
            bones[i].base_t[:] = [float(x) for x in bd["base_t"]]
            bones[i].base_r[:] = [float(x) for x in bd["base_r"]]
            bones[i].base_s[:] = [float(x) for x in bd["base_s"]]
        keep, anims = [], (runtime.SftgAnimationDesc * len(rig["anims"]))()
        for a, an in enumerate(rig["anims"]):
            smp = (runtime.SftgSamplerDesc * len(an["samplers"]))()
            for k, (ins, outs, step) in enumerate(an["samplers"]):
                ia, oa = np.ascontiguousarray(ins, np.float32), np.ascontiguousarray(outs, np.float32)
                keep += [ia, oa]
                smp[k] = runtime.SftgSamplerDesc(ia.ctypes.data, oa.ctypes.data, len(ia), int(step))
            chs = (runtime.SftgChannelDesc * len(an["channels"]))(*[runtime.SftgChannelDesc(*c) for c in an["channels"]])
            keep += [smp, chs]
            anims[a] = runtime.SftgAnimationDesc(C.cast(smp, C.c_void_p), C.cast(chs, C.c_void_p), len(an["samplers"]),
                                                 len(an["channels"]), float(an["duration"]))
        assert L.sft_model_set_skeleton(model, bones, nb, anims, len(rig["anims"])) == 0
        pose = L.sft_pose_create(model, None)
        L.sft_pose_update(pose, 0, C.c_float(0.37))
        ptrs = (C.c_void_p * 3).from_address(pose)   # sft_pose: model, global_matrices, posed_bone_matrices
        glob = np.ctypeslib.as_array((C.c_float * (nb * 16)).from_address(ptrs[1]))
        posed = np.ctypeslib.as_array((C.c_float * (nb * 16)).from_address(ptrs[2]))
        assert np.array_equal(posed, exp) and np.array_equal(glob, exp_g)
        before = posed.copy()
        L.sft_pose_update(pose, 9, C.c_float(0.5))   # no such animation: matrices untouched
        assert np.array_equal(posed, before)
    finally:
        renderer.free_scene(h)
