"""The SoA math helpers of include/sofren2.h (sft_vv_* and sft_vm_broadcast, sofren2.c:780-792,
1921-2060) against the reference's own helpers in its AVX2 build, bit for bit, on seeded groups
of eight lanes: ordinary vectors, zero and tiny vectors (norm's epsilon, RSQRTPS of 0 and of
denormals), huge ones whose products overflow (NaN lanes from inf - inf and 0 * inf, which must
carry x86's default NaN on any host), negative zero, and every RSQRTPS exponent parity.  The reference's
output is pinned by a digest (tests/golden/golden.json, 'soa_math') and, where the reference
is compiled here (oracle/_ref), also compared directly."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import golden_cases as gc
from oracle_lib import REF_DIR

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def soa_inputs(groups: int = 512, seed: int = 7001) -> np.ndarray:
    """groups x [a.xyz (8 each), b.xyz (8 each), s (8), m (16)] as f32."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(-4.0, 4.0, size=(groups, 72)).astype(np.float32)
    mag = np.float32(10.0) ** rng.integers(-20, 20, size=(groups, 1)).astype(np.float32)
    x[:, :24] *= mag                                       # a spans 1e-20 .. 1e19 per group
    x[0:8, :24] = 0.0                                      # zero vectors
    x[8:16, :24] = np.float32(1e-30)                      # |a|^2 is denormal or zero
    x[16:24, :24] = -0.0
    x[24:32, :24] = np.float32(3e18)
    with np.errstate(over="ignore"):
        x[32:40, :48] *= np.float32(1e19)                 # |a|^2, a.b and the cross product overflow:
        x[32:40, 56:72] *= np.float32(1e19)               # inf - inf and 0 * inf give NaN lanes
    return x


def _run(exe: str, inp: np.ndarray, tmp) -> np.ndarray:
    i, o = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    inp.tofile(i)
    subprocess.run([exe, i, o], check=True)
    return np.fromfile(o, np.uint32)


@pytest.fixture(scope="module")
def soa_exe(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path_factory.mktemp("soa") / "soa_math")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=gnu11", "-Wno-psabi", "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "soa_math.c"), "-o", exe, "-lm"], check=True)
    return exe


def test_soa_math_matches_reference_digest(golden, soa_exe, tmp_path):
    out = _run(soa_exe, soa_inputs(), str(tmp_path))
    assert out.size == 512 * 43 * 8
    assert gc.sha(out) == golden["soa_math"]["sha256"]


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_DIR, "soa_harness")),
                    reason="reference not compiled here (oracle/_ref, x86-64 with AVX2)")
def test_soa_math_equals_reference(soa_exe, tmp_path):
    inp = soa_inputs(groups=2048, seed=7002)
    ours = _run(soa_exe, inp, str(tmp_path))
    ref = _run(os.path.join(REF_DIR, "soa_harness"), inp, str(tmp_path))
    bad = np.nonzero(ours != ref)[0]
    assert bad.size == 0, f"{bad.size} words differ, first at {bad[:8].tolist()}"
