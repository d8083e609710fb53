"""Batched rendering: many scenes in one wavefront (shared pass queues, one captured
pass replayed as a CUDA graph, launch shape picked by timing candidates). Each scene's
image must equal its own single-scene render with the same options: the random-number
keys are per scene and per path, so the two differ only by the summation order of the
FP64 film."""
import numpy as np
import pytest

import renderx_gb300 as rx
from renderx_gb300 import scenes

pytestmark = pytest.mark.gpu


def _scenes():
    return [(scenes.cornell_box(32, 32), dict(spp=64, max_depth=8, rr_mode=0, nee=False, seed=11)),
            (scenes.material_spheres(48, 32), dict(spp=32, max_depth=8, rr_mode=0, nee=True, seed=12)),
            (scenes.medium_scene(32, 32), dict(spp=48, max_depth=8, rr_mode=1, nee=False, seed=13)),
            (scenes.sphere_field(12, 3, 4, 40, 24), dict(spp=40, max_depth=16, rr_mode=1, nee=True, seed=14))]


@pytest.mark.parametrize("use_graph,autotune", [(True, False), (False, False), (True, True)])
def test_batch_equals_single_scene_renders(use_graph, autotune):
    items = _scenes()
    ctxs = []
    try:
        for sc, _ in items:
            c = rx.Context(0)
            c.set_scene(sc)
            c.build_accel()
            ctxs.append(c)
        singles = [c.render_pt(sc.camera, o["spp"], max_depth=o["max_depth"], nee=o["nee"], rr_mode=o["rr_mode"],
                               seed=o["seed"], paths_per_pass=1 << 13)[0] for c, (sc, o) in zip(ctxs, items)]
        films, st = ctxs[0].render_pt_batch([(c, sc.camera, o) for c, (sc, o) in zip(ctxs, items)],
                                            paths_per_pass=1 << 13, use_graph=use_graph, autotune=autotune)
    finally:
        for c in ctxs:
            c.close()
    for a, b in zip(films, singles):
        assert a.shape == b.shape
        assert np.allclose(a, b, rtol=1e-9, atol=1e-12), np.abs(a - b).max()
        assert a.mean() > 0
    assert st["paths"] == sum(sc.camera.width * sc.camera.height * o["spp"] for sc, o in items)
    assert st["blocks_per_sm"] in (4, 8, 16) and st["stack"] in (4, 5, 32, 64)


def test_batch_rejects_bad_input():
    sc = scenes.cornell_box(16, 16)
    with rx.Context(0) as c, rx.Context(0) as bare:
        c.set_scene(sc)
        c.build_accel()
        with pytest.raises(rx.RxError):
            c.render_pt_batch([])
        with pytest.raises(rx.RxError):
            c.render_pt_batch([(bare, sc.camera, dict(spp=4))])
        with pytest.raises(rx.RxError):
            c.render_pt_batch([(c, sc.camera, dict(spp=0))])
