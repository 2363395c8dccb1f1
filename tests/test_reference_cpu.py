"""The reference's own CPU build on this host, the one bench.py times as its CPU baseline
(oracle/_ref/ref_bench_*, `make -C oracle ref_bench`: the NEON path, 4 lanes, on an aarch64 host;
AVX2 with GCC's default contraction on x86-64), renders the benchmark's scenes, and its frames
agree with the oracle's (which equal the GPU's bit for bit): so the baseline does the same work.
Its bits are not the parity target (other SIMD width, other reciprocal estimates, contracted
multiply-adds), so the check is the tolerance bench.py applies before it times the build: most
pixels within a few LSB per channel and a small mean difference.
Skipped where that build is absent."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from oracle_io import read_dump
from oracle_lib import REF_DIR


def _ref_color(blob: bytes, samples: int, frame: int = 0) -> np.ndarray:
    exe = os.path.join(REF_DIR, f"ref_bench_{samples}x")
    if not os.path.exists(exe):
        pytest.skip("the reference's own CPU build is absent on this host")
    with tempfile.TemporaryDirectory() as td:
        sp, dp = os.path.join(td, "s.sfts"), os.path.join(td, "r.dump")
        open(sp, "wb").write(blob)
        subprocess.run([exe, sp, dp, str(frame), str(os.cpu_count() or 1)], check=True, stdout=subprocess.DEVNULL)
        return read_dump(dp)[0]["color"]


@pytest.mark.parametrize("gen, samples", [("config1", 1), ("config2", 2)])
def test_reference_cpu_build_renders_the_bench_scene(gen, samples):
    from oracle_lib import Oracle
    from sofren2_gb300 import scenes
    sc = getattr(scenes, gen)()
    blob = sc.to_bytes()
    f = sc.frames[0]
    ref = _ref_color(blob, samples).reshape(f.height, f.width)
    o = Oracle(blob)
    try:
        ours, _, _ = o.render_color(0, samples, f.width, f.height, threads=os.cpu_count() or 1)
    finally:
        o.close()
    ours = ours.reshape(f.height, f.width)
    a = np.stack([(ref >> s) & 0xFF for s in (16, 8, 0)]).astype(np.int32)
    b = np.stack([(ours >> s) & 0xFF for s in (16, 8, 0)]).astype(np.int32)
    d = np.abs(a - b).max(axis=0)
    close = float((d <= 4).mean())
    print(f"{gen}: {close:.5f} of pixels within 4 LSB, mean |d| {np.abs(a - b).mean():.4f}")
    import bench
    assert close >= bench.REF_AGREEMENT_MIN, f"{gen}: only {close:.4f} of pixels within 4 LSB of the oracle's frame"
    assert np.abs(a - b).mean() <= bench.REF_MEAN_LSB_MAX
