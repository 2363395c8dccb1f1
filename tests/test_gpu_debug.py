"""Debug views on the GPU (wireframe, tile grid, depth, light count, checkerboard) against the
reference's own renders of the same views, single frames and batched."""
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", gc.DEBUG_CASES, ids=lambda c: f"{c[0]}-{c[1]}-{c[2]}x")
def test_debug_view_matches_reference(renderer, golden, case):
    name, mode, S = case
    h = renderer.load_scene(gc.blob(name))
    try:
        renderer.set_samples(S)
        renderer.set_debug_mode(mode)
        c = renderer.render(h, 0)
    finally:
        renderer.set_debug_mode(0)
        renderer.set_samples(1)
        renderer.free_scene(h)
    assert gc.sha(c.reshape(-1)) == golden["debug_views"][f"{name}/{mode}/{S}"]


@pytest.mark.parametrize("mode", [1, 2, 3, 4, 5])
def test_debug_views_batched(renderer, golden, mode):
    cases = [c for c in gc.DEBUG_CASES if c[1] == mode]
    names = sorted({n for n, _, _ in cases})
    hs = {n: renderer.load_scene(gc.blob(n)) for n in names}
    try:
        renderer.set_debug_mode(mode)
        got = renderer.render_batch([(hs[n], 0, S) for n, _, S in cases], [None] * len(cases))
    finally:
        renderer.set_debug_mode(0)
        for h in hs.values():
            renderer.free_scene(h)
    for (n, m, S), c in zip(cases, got):
        assert gc.sha(c.reshape(-1)) == golden["debug_views"][f"{n}/{m}/{S}"], f"{n} view {m} {S}x differs in a batch"
