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
                                            paths_per_pass=1 << 12, use_graph=use_graph, autotune=autotune)
    finally:
        for c in ctxs:
            c.close()
    for a, b in zip(films, singles):
        assert a.shape == b.shape
        assert np.allclose(a, b, rtol=1e-9, atol=1e-12), np.abs(a - b).max()
        assert a.mean() > 0
    assert st["paths"] == sum(sc.camera.width * sc.camera.height * o["spp"] for sc, o in items)
    assert st["blocks_per_sm"] in (4, 8, 16) and st["stack"] in (4, 5, 6, 32, 64)


def test_autotuned_batch_picks_a_pass_size_and_equals_single_scene_renders():
    """Autotuning times the launch shapes and then the pass sizes 2^20..2^23 (two passes
    each, on interleaved passes that hold the same mix of every scene); the remaining
    passes take the scenes one after another, each continuing after the paths the
    tuning took from it. The chosen size is reported, and every image still equals its
    single-scene render up to the FP64 summation order (the random numbers depend on
    each scene's own path indices only)."""
    items = [(scenes.cornell_box(128, 128), dict(spp=512, max_depth=8, rr_mode=1, seed=31)),
             (scenes.material_spheres(128, 128), dict(spp=512, max_depth=8, rr_mode=1, seed=32)),
             (scenes.medium_scene(128, 128), dict(spp=512, max_depth=8, rr_mode=1, seed=33)),
             (scenes.cornell_box(128, 128), dict(spp=512, max_depth=8, rr_mode=0, nee=True, seed=34))]
    ctxs = []
    try:
        for sc, _ in items:
            c = rx.Context(0)
            c.set_scene(sc)
            c.build_accel()
            ctxs.append(c)
        singles = [c.render_pt(sc.camera, o["spp"], max_depth=o["max_depth"], nee=o.get("nee", False),
                               rr_mode=o["rr_mode"], seed=o["seed"])[0] for c, (sc, o) in zip(ctxs, items)]
        films, st = ctxs[0].render_pt_batch([(c, sc.camera, o) for c, (sc, o) in zip(ctxs, items)],
                                            paths_per_pass=1 << 18, autotune=True)
    finally:
        for c in ctxs:
            c.close()
    total = sum(sc.camera.width * sc.camera.height * o["spp"] for sc, o in items)
    assert st["paths"] == total
    assert st["paths_per_pass"] in [sum(-(-128 * 128 * 512 * sz // total) for _ in items)
                                    for sz in (1 << 20, 1 << 21, 1 << 22)], st["paths_per_pass"]
    for a, b in zip(films, singles):
        assert np.allclose(a, b, rtol=1e-9, atol=1e-12), np.abs(a - b).max()


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


def test_guided_batch_is_unbiased_and_leaves_plain_items_unchanged():
    """One batch with three guided scenes (two glossy sphere fields and the Cornell box,
    each with its own network, trained during the render) and one plain scene. Each
    guided image, averaged over independent batch renders (networks re-initialised for
    each), agrees per pixel with a high-sample plain render of its scene within 3 sigma
    (at most 2% of channels, none beyond 8 sigma; image means within 4 standard errors):
    the grouped inference and per-network training change the sampling density, never
    the estimator's expectation. The plain item, whose random numbers depend only on its
    own path indices, equals its single-scene render up to the FP64 summation order."""
    guided = [(scenes.guiding_scene(40, 40, n_spheres=20, subdiv=2, seed=3), 8),
              (scenes.guiding_scene(32, 32, n_spheres=30, subdiv=2, seed=4), 8),
              (scenes.cornell_box(32, 32), 8)]
    plain_sc, plain_o = scenes.material_spheres(32, 24), dict(spp=64, max_depth=8, rr_mode=0, nee=True, seed=21)
    runs, spp, ref_spp = 24, 512, 32768
    ctxs = []
    try:
        for sc, _ in guided + [(plain_sc, 0)]:
            c = rx.Context(0)
            c.set_scene(sc)
            c.build_accel()
            ctxs.append(c)
        refs = []
        for c, (sc, depth) in zip(ctxs, guided):
            m, sq, _ = c.render_pt(sc.camera, ref_spp, max_depth=depth, rr_mode=1, seed=7, want_sq=True)
            refs.append((m, np.sqrt(np.maximum(sq - m * m, 0.0) / (ref_spp - 1))))
        single = ctxs[3].render_pt(plain_sc.camera, plain_o["spp"], max_depth=8, nee=True, rr_mode=0,
                                   seed=plain_o["seed"], paths_per_pass=1 << 13)[0]
        imgs = [[] for _ in guided]
        for r in range(runs):
            for k, c in enumerate(ctxs[:3]):
                c.guide_init(seed=100 * r + k, batch=1 << 14, warmup_passes=2, train_passes=6, steps_per_pass=4)
            items = [(c, sc.camera, dict(spp=spp, max_depth=depth, rr_mode=1, seed=1000 + 10 * r + k, guided=True))
                     for k, (c, (sc, depth)) in enumerate(zip(ctxs, guided))]
            items.append((ctxs[3], plain_sc.camera, plain_o))
            films, st = ctxs[0].render_pt_batch(items, paths_per_pass=1 << 16, use_graph=True, autotune=(r == 0))
            for k in range(3):
                imgs[k].append(films[k])
            assert np.allclose(films[3], single, rtol=1e-9, atol=1e-12), np.abs(films[3] - single).max()
    finally:
        for c in ctxs:
            c.close()
    for k, (ref, rse) in enumerate(refs):
        a = np.array(imgs[k])
        mean = a.mean(axis=0)
        se = a.std(axis=0, ddof=1) / np.sqrt(runs)
        sig = np.sqrt(se ** 2 + rse ** 2)
        zz = np.abs(mean - ref) / (sig + 1e-12)
        bad = np.abs(mean - ref) > 3 * sig + 1e-4
        assert bad.mean() <= 0.02, f"scene {k}: {bad.mean():.4f} beyond 3 sigma (max z {zz.max():.1f})"
        assert (zz > 8).sum() == 0, f"scene {k}: max z {zz.max():.1f}"
        n = mean.shape[0] * mean.shape[1]
        for ch in range(3):
            dm = mean[..., ch].mean() - ref[..., ch].mean()
            s_img = np.sqrt((se[..., ch] ** 2).sum() + (rse[..., ch] ** 2).sum()) / n
            assert abs(dm) < 4 * s_img, (k, ch, dm, s_img)


def test_guided_batch_trains_each_scene_network():
    """Each guided item's network is trained on its own scene's records: after the
    render every network differs from its initial weights, and networks initialised
    alike but serving different scenes end up different."""
    scs = [scenes.guiding_scene(32, 32, n_spheres=20, subdiv=2, seed=5), scenes.cornell_box(32, 32)]
    ctxs = []
    try:
        for sc in scs:
            c = rx.Context(0)
            c.set_scene(sc)
            c.build_accel()
            c.guide_init(seed=9, batch=1 << 13, warmup_passes=1, train_passes=4, steps_per_pass=2,
                         box=((0.0, 0.0, 0.0), (5.56, 5.56, 5.56)))
            ctxs.append(c)
        p0 = [c.guide_params() for c in ctxs]
        assert np.array_equal(p0[0], p0[1])
        items = [(c, sc.camera, dict(spp=256, max_depth=8, rr_mode=1, seed=3, guided=True)) for c, sc in zip(ctxs, scs)]
        films, _ = ctxs[0].render_pt_batch(items, paths_per_pass=1 << 15)
        p1 = [c.guide_params() for c in ctxs]
    finally:
        for c in ctxs:
            c.close()
    for a, b in zip(p0, p1):
        assert not np.array_equal(a, b)
        assert np.isfinite(b).all()
    assert not np.array_equal(p1[0], p1[1])
    assert all(f.mean() > 0 and np.isfinite(f).all() for f in films)


def test_guided_batch_rejects_items_without_network_or_with_light_sampling():
    sc = scenes.cornell_box(16, 16)
    with rx.Context(0) as c:
        c.set_scene(sc)
        c.build_accel()
        with pytest.raises(rx.RxError, match="rx_guide_init"):
            c.render_pt_batch([(c, sc.camera, dict(spp=4, guided=True))])
        c.guide_init(seed=1)
        with pytest.raises(rx.RxError, match="nee"):
            c.render_pt_batch([(c, sc.camera, dict(spp=4, nee=True, guided=True))])
        films, _ = c.render_pt_batch([(c, sc.camera, dict(spp=64, guided=True))], paths_per_pass=1 << 12)
        assert films[0].mean() > 0
