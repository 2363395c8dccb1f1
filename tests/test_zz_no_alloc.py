"""sftg_light_vis_noalloc, the allocation-free light-visibility entry point, called through the C
ABI: two calls in a row give the light_vis rows that sftg_frame_render computes for the same
frame, and a frame too large for the static scratch is refused before any device work.

Named to be collected last, so it also runs after every other GPU test in the session."""
import ctypes as C
import os

import numpy as np
import pytest

import golden_cases as gc
from sofren2_gb300 import runtime

pytestmark = pytest.mark.gpu

SFTG_E_LIMIT = -4


class FrameDescHead(C.Structure):
    """Leading fields of struct sftg_frame_desc (include/sftg.h), up to n_proxies."""
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("samples", C.c_int32), ("cam_pos", C.c_float * 3),
        ("view_proj", C.c_float * 16), ("frustum_n", C.c_float * 18), ("frustum_d", C.c_float * 6),
        ("ambient", C.c_float * 3), ("lightmap_brightness", C.c_float),
        ("clear", C.c_uint32), ("clear_color", C.c_uint32), ("shadows", C.c_uint32), ("debug_mode", C.c_uint32),
        ("n_point", C.c_uint32), ("point_lights", C.c_void_p), ("n_dir", C.c_uint32), ("dir_lights", C.c_void_p),
        ("n_instances", C.c_uint32), ("instances", C.c_void_p), ("n_proxies", C.c_uint32), ("proxies", C.c_void_p),
        ("tlas_nodes", C.c_void_p), ("tlas_count", C.c_uint32), ("tlas_root", C.c_uint32),
    ]


@pytest.fixture(scope="module")
def lib(renderer):
    L = renderer.lib
    L.sft_batch_begin.restype, L.sft_batch_begin.argtypes = None, []
    L.sft_batch_submit.restype, L.sft_batch_submit.argtypes = C.c_int32, []
    L.sft_batch_peek.restype, L.sft_batch_peek.argtypes = C.c_void_p, [C.c_uint32]
    L.sft_get_gpu_context.restype, L.sft_get_gpu_context.argtypes = C.c_void_p, []
    L.sftg_light_vis_noalloc.restype = C.c_int
    L.sftg_light_vis_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.sftg_frame_render.restype = C.c_int
    L.sftg_frame_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
    L.sftg_last_error.restype, L.sftg_last_error.argtypes = C.c_char_p, [C.c_void_p]
    return L


def _device_free_bytes() -> int:
    """cudaMemGetInfo's free bytes through the CUDA runtime the library itself loaded (found by
    its soname among the process's loaded libraries, not loaded a second time)."""
    rt = C.CDLL("libcudart.so.13", mode=os.RTLD_NOLOAD | os.RTLD_GLOBAL)
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def _recorded_frame(renderer, lib, h):
    """Records frame 0 of a loaded scene with sft_batch_begin and returns its sftg_frame_desc."""
    lib.sft_batch_begin()
    assert renderer.lib.sftx_scene_render(h, 0, None, 0) == 0
    fd = lib.sft_batch_peek(0)
    assert fd
    return fd


@pytest.mark.parametrize("name", ["atrium_small", "variety", "config1"])
def test_noalloc_matches_frame_render(renderer, lib, name):
    h = renderer.load_scene(gc.blob(name))
    renderer.set_samples(1)
    try:
        fd = _recorded_frame(renderer, lib, h)
        ctx = lib.sft_get_gpu_context()
        n_prox = C.cast(fd, C.POINTER(FrameDescHead)).contents.n_proxies
        assert n_prox > 0
        ref = np.zeros(n_prox * 64, np.uint8)
        dbg = runtime.SftgDebugOut()
        dbg.light_vis = ref.ctypes.data
        rc = lib.sftg_frame_render(ctx, fd, None, 0, C.byref(dbg))
        assert rc == 0, lib.sftg_last_error(ctx)
        outs, free = [], [_device_free_bytes()]
        for _ in range(2):
            out = np.full(n_prox * 64, 0xAB, np.uint8)
            rc = lib.sftg_light_vis_noalloc(ctx, fd, out.ctypes.data)
            assert rc == 0, lib.sftg_last_error(ctx)
            outs.append(out)
            free.append(_device_free_bytes())
        # the contract itself: the calls take no device memory (the scratch was committed when
        # the context was created, so not even the first call changes the free bytes)
        assert free[0] == free[1] == free[2], f"{name}: device free memory changed across the calls: {free}"
        assert np.array_equal(outs[0], ref), f"{name}: first allocation-free call differs from sftg_frame_render"
        assert np.array_equal(outs[1], ref), f"{name}: second allocation-free call differs from sftg_frame_render"
        lights = gc.n_lights(name)
        assert np.all(ref.reshape(-1, 64)[:, lights:] == 0)
    finally:
        lib.sft_batch_submit()
        renderer.free_scene(h)


def test_noalloc_rejects_frames_beyond_scratch(renderer, lib):
    h = renderer.load_scene(gc.blob("atrium_small"))
    try:
        renderer.render(h, 0)   # puts the freshly uploaded model table on the device
        fd = _recorded_frame(renderer, lib, h)
        ctx = lib.sft_get_gpu_context()
        big = FrameDescHead.from_buffer_copy(C.string_at(fd, C.sizeof(FrameDescHead)))
        # 64 lights x 4096 proxies: far more packets than the static scratch holds; refused on
        # the host from the counts alone, before any array is read
        big.n_point, big.n_proxies, big.shadows = 64, 4096, 1
        out = np.zeros(16, np.uint8)
        rc = lib.sftg_light_vis_noalloc(ctx, C.byref(big), out.ctypes.data)
        assert rc == SFTG_E_LIMIT
        assert b"static scratch" in lib.sftg_last_error(ctx)
    finally:
        lib.sft_batch_submit()
        renderer.free_scene(h)
