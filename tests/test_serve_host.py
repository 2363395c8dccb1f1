"""The serving loop's host logic (sofren2_gb300/csrc/sft_serve.c, compiled unchanged) on the CPU,
against fakes of the library calls it makes (tests/serve_fake.c): admission within the batch size
and the device-memory budget (counted over every batch in flight), a request larger than the
budget served alone, no more than `lanes` batches in flight and never two on one lane, failed
renders, submissions and waits counted without stopping the loop, arrivals honoured, and the
argument checks; and the warm-up that grows every lane with the largest admissible batch before a
run.  No GPU is involved."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REQ = np.dtype([("arrival_ns", "<u8"), ("device_bytes", "<u8"), ("scene", "<u4"), ("frame", "<u4"),
                ("samples", "<i4"), ("max_point_lights", "<u4")])
BATCHED, PLAIN, OVERLAP = 0, 1, 2
NONE = 0xFFFFFFFF


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    so = str(tmp_path_factory.mktemp("serve") / "libservefake.so")
    subprocess.run([cc, "-O2", "-std=gnu11", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "sofren2_gb300", "csrc", "sft_serve.c"), os.path.join(ROOT, "tests", "serve_fake.c"),
                    "-o", so], check=True)
    L = C.CDLL(so)
    p, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
    L.sftx_serve_ex.restype = C.c_int
    L.sftx_serve_ex.argtypes = [p, p, u32, u32, u64, C.c_int, u32, p, u32, p, p, p]
    L.sftx_serve_warm.restype = C.c_int
    L.sftx_serve_warm.argtypes = [p, p, u32, u32, u64, u32, p, u32]
    L.fk_reset.argtypes = [u32, u32, u32, u32]
    L.fk_stats.argtypes = [p]
    L.fk_batch_size.restype, L.fk_batch_size.argtypes = u32, [u32]
    return L


def serve(L, reqs, max_batch, budget, mode, lanes=3, n_colors=None, polls=3, fail=(NONE, NONE, NONE)):
    n = len(reqs)
    n_colors = n_colors or max_batch
    bufs = [np.zeros(4, np.uint32) for _ in range(n_colors)]
    colors = (C.c_void_p * n_colors)(*[b.ctypes.data for b in bufs])
    scenes = (C.c_void_p * 4)(*[C.c_void_p(0x1000 * (k + 1)) for k in range(4)])
    r = np.ascontiguousarray(reqs, REQ)
    done = np.zeros(max(1, n), np.uint64)
    batch_of = np.full(max(1, n), NONE, np.uint32)
    stats = np.zeros(5, np.uint64)
    L.fk_reset(polls, *fail)
    rc = L.sftx_serve_ex(scenes, r.ctypes.data, n, max_batch, budget, mode, lanes, colors, n_colors, done.ctypes.data,
                         batch_of.ctypes.data, stats.ctypes.data)
    fk = np.zeros(6, np.uint32)
    L.fk_stats(fk.ctypes.data)
    sizes = [L.fk_batch_size(i) for i in range(int(fk[5]))]
    names = ("batches", "max_batch", "peak_bytes", "errors", "max_inflight")
    return rc, dict(zip(names, map(int, stats))), dict(zip(("renders", "submits", "waits", "busy_submit", "max_busy", "nbatches"),
                                                          map(int, fk))), sizes, done[:n], batch_of[:n]


def requests(n, bytes_each=10, gap_ns=0):
    r = np.zeros(n, REQ)
    r["arrival_ns"] = np.arange(n, dtype=np.uint64) * gap_ns
    r["device_bytes"] = bytes_each
    r["scene"] = np.arange(n) % 4
    r["frame"] = np.arange(n)
    r["samples"] = 1
    r["max_point_lights"] = 64
    return r


def test_overlap_within_lanes_budget_and_batch(lib):
    # budget-bound: ten 10-byte requests fill the 100-byte budget, so one batch at a time
    rc, st, fk, sizes, done, batch_of = serve(lib, requests(200), max_batch=16, budget=100, mode=OVERLAP, lanes=3, n_colors=64)
    assert rc == 0 and st["errors"] == 0
    assert sum(sizes) == 200 and fk["renders"] == 200
    assert max(sizes) == 10 and st["max_batch"] == 10 and st["peak_bytes"] <= 100
    assert st["max_inflight"] == 1 and fk["busy_submit"] == 0
    assert (batch_of != NONE).all() and (np.diff(batch_of.astype(np.int64)) >= 0).all()
    # lane-bound: every lane busy, never more, never two batches on one lane
    rc, st, fk, sizes, done, batch_of = serve(lib, requests(200), max_batch=4, budget=1 << 30, mode=OVERLAP, lanes=3, n_colors=64)
    assert rc == 0 and sum(sizes) == 200 and max(sizes) <= 4
    assert st["max_inflight"] == 3 and fk["max_busy"] == 3 and fk["busy_submit"] == 0
    assert st["peak_bytes"] == 120                               # three batches of 40 bytes in flight
    # the budget counts every batch in flight: with 100 bytes, two batches of 4 leave room for a
    # batch of 2 beside them, never more
    rc, st, fk, sizes, done, batch_of = serve(lib, requests(200), max_batch=4, budget=100, mode=OVERLAP, lanes=3, n_colors=64)
    assert rc == 0 and sum(sizes) == 200
    assert st["peak_bytes"] == 100 and min(sizes) < 4 and fk["max_busy"] <= 3 and fk["busy_submit"] == 0


def test_request_larger_than_budget_served_alone(lib):
    r = requests(5)
    r["device_bytes"] = [10, 10, 500, 10, 10]
    for mode in (OVERLAP, BATCHED):
        rc, st, fk, sizes, done, batch_of = serve(lib, r, max_batch=4, budget=100, mode=mode)
        assert rc == 0 and sum(sizes) == 5
        assert (batch_of == batch_of[2]).sum() == 1, f"mode {mode}: the oversize request shares its batch"


def test_failures_counted_and_loop_finishes(lib):
    rc, st, fk, sizes, done, batch_of = serve(lib, requests(60), max_batch=8, budget=1 << 30, mode=OVERLAP, lanes=2,
                                              n_colors=16, fail=(5, 2, 1))
    assert rc == -2 and st["errors"] == 3
    assert sum(sizes) == 60 and (batch_of != NONE).all()
    rc, st, fk, sizes, done, batch_of = serve(lib, requests(30), max_batch=8, budget=1 << 30, mode=BATCHED, fail=(3, 1, NONE))
    assert rc == -2 and st["errors"] == 2 and sum(sizes) == 30


def test_batched_and_plain_modes(lib):
    rc, st, fk, sizes, done, batch_of = serve(lib, requests(40), max_batch=8, budget=1 << 30, mode=BATCHED)
    assert rc == 0 and fk["max_busy"] == 0 and sum(sizes) == 40 and max(sizes) <= 8
    rc, st, fk, sizes, done, batch_of = serve(lib, requests(40), max_batch=8, budget=1 << 30, mode=PLAIN)
    assert rc == 0 and fk["nbatches"] == 0 and fk["renders"] == 40 and st["batches"] == 40


def test_arrivals_are_honoured(lib):
    r = requests(30, gap_ns=1_000_000)
    for mode in (OVERLAP, BATCHED, PLAIN):
        rc, st, fk, sizes, done, batch_of = serve(lib, r, max_batch=4, budget=1 << 30, mode=mode)
        assert rc == 0
        assert (done >= r["arrival_ns"]).all(), f"mode {mode}: a request completed before it arrived"


def test_argument_checks(lib):
    r = requests(4)
    assert serve(lib, r, max_batch=4, budget=100, mode=OVERLAP, n_colors=2)[0] == -1   # fewer colour buffers than a batch
    assert serve(lib, r, max_batch=4, budget=100, mode=OVERLAP, lanes=0)[0] == -1
    assert serve(lib, r, max_batch=4, budget=100, mode=OVERLAP, lanes=8)[0] == -1
    assert serve(lib, r, max_batch=4, budget=100, mode=7)[0] == -1


def warm(L, reqs, max_batch, budget, lanes, n_colors=None, fail=(NONE, NONE, NONE)):
    n_colors = n_colors or max_batch
    bufs = [np.zeros(4, np.uint32) for _ in range(n_colors)]
    colors = (C.c_void_p * n_colors)(*[b.ctypes.data for b in bufs])
    scenes = (C.c_void_p * 4)(*[C.c_void_p(0x1000 * (k + 1)) for k in range(4)])
    r = np.ascontiguousarray(reqs, REQ)
    L.fk_reset(3, *fail)
    rc = L.sftx_serve_warm(scenes, r.ctypes.data, len(r), max_batch, budget, lanes, colors, n_colors)
    fk = np.zeros(6, np.uint32)
    L.fk_stats(fk.ctypes.data)
    stats = dict(zip(("renders", "submits", "waits", "busy_submit", "max_busy", "nbatches"), map(int, fk)))
    return rc, stats, [L.fk_batch_size(i) for i in range(stats["nbatches"])], [int(b[0]) for b in bufs]


def test_warm_renders_the_largest_batch_on_every_lane(lib):
    r = requests(50)
    r["device_bytes"][[7, 20, 33, 41, 45]] = [50, 40, 40, 30, 30]   # ties go to the earlier request
    rc, fk, sizes, firsts = warm(lib, r, max_batch=4, budget=1 << 30, lanes=3, n_colors=6)
    assert rc == 0
    assert sizes == [4, 4, 4, 4]                       # lanes 1-3, then lane 0
    assert fk["max_busy"] == 3 and fk["busy_submit"] == 0 and fk["waits"] == 3
    assert firsts[:4] == [8, 21, 34, 42]               # frame + 1 of requests 7, 20, 33, 41, largest first
    # within the budget, largest first; a request over the budget on its own still warms alone
    assert warm(lib, r, max_batch=4, budget=100, lanes=2)[2] == [2, 2, 2]
    assert warm(lib, r, max_batch=4, budget=10, lanes=1)[2] == [1, 1]
    # lane 0 only
    rc, fk, sizes, _ = warm(lib, r, max_batch=8, budget=1 << 30, lanes=0)
    assert rc == 0 and sizes == [8] and fk["waits"] == 0


def test_warm_failures_and_argument_checks(lib):
    r = requests(10)
    assert warm(lib, r, max_batch=4, budget=1 << 30, lanes=2, fail=(5, NONE, NONE))[0] == -2
    assert warm(lib, r, max_batch=4, budget=1 << 30, lanes=2, fail=(NONE, NONE, 1))[0] == -2
    assert warm(lib, r, max_batch=4, budget=1 << 30, lanes=2, n_colors=3)[0] == -1
    assert warm(lib, r, max_batch=4, budget=1 << 30, lanes=8)[0] == -1
    assert warm(lib, r[:0], max_batch=4, budget=1 << 30, lanes=2)[0] == -1
