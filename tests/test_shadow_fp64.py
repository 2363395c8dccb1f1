"""The capsule shadow expression (sofren2.c:6522-6571) in FP32 against an FP64 evaluation of the
same expression, on the CPU.  The FP32 values are the oracle's, which equal the reference's bit for
bit (and the GPU's: colour is bit-exact on every golden case); the FP64 evaluation
(sfto_shadow_fp64) recomputes every quantity in double from the pixel positions, the light and the
proxies' endpoints, with the same proxies, gates, block-level skip and smooth maximum.

What is measured: away from gate boundaries the FP32 shadow intensity is within about 1.5e-5 of
the FP64 one (the table reciprocal and the fast normalisation dominate).  At a boundary a proxy
can count as active for a 4x2 block in one precision and not in the other; the reference's
block-level rule then adds the smooth maximum's blend term (up to 0.2^2 x 1.25 = 0.05) to every
lane of the block, which is what the atrium's few larger differences are."""
import pytest

import golden_cases as gc
from oracle_lib import Oracle


@pytest.mark.parametrize("name, samples, worst", [
    ("skinned_small", 1, 5e-5),
    ("variety", 1, 1e-6),
    ("atrium_small", 1, 0.0501),
    ("atrium_small", 4, 0.0501),
])
def test_fp32_shadow_against_fp64(name, samples, worst):
    r = Oracle(gc.blob(name)).shadow_fp64(0, samples)
    print(f"{name} {samples}x: max {r['max']:.3g}, mean {r['mean']:.3g}, {r['over_1e-5']} of {r['n']} over 1e-5")
    assert r["n"] > 10000, "the case must exercise the shadow loop"
    assert r["max"] <= worst
    assert r["mean"] < 1e-6
    assert r["over_1e-5"] <= r["n"] * 2e-4
