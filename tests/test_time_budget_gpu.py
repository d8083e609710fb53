"""Time budgets (the reference's <time> runtime: MCRenderer::runtime, checked after each
iteration in PathTracer.cpp:87, VCMTracer.cpp:142, BidirectionalPathTracer.cpp:114). A
budget far below one pass stops the render at the second path-tracing pass (the check
after queueing pass p waits for pass p - 1) or after the first iteration of the
iterative estimators; the random numbers are keyed by path and iteration only, so the
result must equal the fixed-count render with the same seed up to summation order: of
the FP64 film for path tracing (rtol 1e-9), of each iteration's FP32 image atomics for
the iterative estimators (rtol 1e-5, atol 1e-6 of the image maximum)."""
import numpy as np
import pytest

import renderx_gb300 as rx
from renderx_gb300 import scenes

pytestmark = pytest.mark.gpu
TINY = 1e-6  # seconds: spent before any pass completes


def _ctx(sc):
    c = rx.Context(0)
    c.set_scene(sc)
    c.build_accel()
    return c


def test_pt_budget_stops_on_whole_samples():
    sc = scenes.cornell_box(64, 64)
    n = 64 * 64
    with _ctx(sc) as c:
        img, _, st = c.render_pt(sc.camera, 200, max_depth=8, seed=5, paths_per_pass=n, time_budget_s=TINY)
        ref, _, st2 = c.render_pt(sc.camera, 2, max_depth=8, seed=5, paths_per_pass=n)
    assert st["paths"] == 2 * n and st2["paths"] == 2 * n
    assert np.allclose(img, ref, rtol=1e-9, atol=1e-12)
    assert img.mean() > 0


def test_pt_budget_mid_sample_normalises_each_pixel_by_its_own_count():
    sc = scenes.cornell_box(64, 64)
    n, per = 64 * 64, 3000
    with _ctx(sc) as c:
        img, _, st = c.render_pt(sc.camera, 100, max_depth=8, nee=True, seed=9, paths_per_pass=per,
                                 time_budget_s=TINY)
        one, _, _ = c.render_pt(sc.camera, 1, max_depth=8, nee=True, seed=9)
        two, _, _ = c.render_pt(sc.camera, 2, max_depth=8, nee=True, seed=9)
    done = 2 * per  # sample-major: pixels below done - n hold two samples, the rest one
    assert st["paths"] == done
    q = np.arange(n).reshape(64, 64)[..., None]
    expect = np.where(q < done - n, two, one)
    assert np.allclose(img, expect, rtol=1e-9, atol=1e-12)


def test_iterative_estimators_stop_after_the_first_iteration():
    sc = scenes.cornell_box(32, 32)
    n = 32 * 32
    with _ctx(sc) as c:
        v, sv = c.render_vcm(sc.camera, 50, 0.1, max_depth=8, seed=3, time_budget_s=TINY)
        v1, _ = c.render_vcm(sc.camera, 1, 0.1, max_depth=8, seed=3)
        b, sb = c.render_bpt(sc.camera, 50, max_depth=8, seed=4, time_budget_s=TINY)
        b1, _ = c.render_bpt(sc.camera, 1, max_depth=8, seed=4)
        p, sp = c.render_pm(sc.camera, 50, 0.1, max_depth=8, seed=6, time_budget_s=TINY)
        p1, _ = c.render_pm(sc.camera, 1, 0.1, max_depth=8, seed=6)
    for img, ref, st in ((v, v1, sv), (b, b1, sb), (p, p1, sp)):
        assert st["paths"] == n
        np.testing.assert_allclose(img, ref, rtol=1e-5, atol=1e-6 * ref.max())
        assert img.mean() > 0


def test_budget_rejects_negative_values():
    sc = scenes.cornell_box(16, 16)
    with _ctx(sc) as c:
        with pytest.raises(rx.RxError):
            c.render_pt(sc.camera, 4, time_budget_s=-1.0)
        with pytest.raises(rx.RxError):
            c.render_vcm(sc.camera, 2, 0.1, time_budget_s=-1.0)
        with pytest.raises(rx.RxError):
            c.render_bpt(sc.camera, 2, time_budget_s=-1.0)
        with pytest.raises(rx.RxError):
            c.render_pm(sc.camera, 2, 0.1, time_budget_s=-1.0)


def test_snapshots_hand_over_the_running_mean():
    # MCRenderer::showCurrentResult(pixelColors, &time, &iter) every timeStep seconds:
    # with a step far below one pass, one snapshot per pass / iteration, each equal to
    # the fixed-count render of that many samples
    sc = scenes.cornell_box(32, 32)
    n = 32 * 32
    got = []
    with _ctx(sc) as c:
        c.set_snapshots(1e-9, lambda t, s, img: got.append((t, s, img)))
        c.render_pt(sc.camera, 3, max_depth=8, seed=5, paths_per_pass=n)
        pt = list(got)
        got.clear()
        c.render_vcm(sc.camera, 3, 0.1, max_depth=8, seed=3)
        vcm = list(got)
        c.set_snapshots(0)
        got.clear()
        c.render_pt(sc.camera, 2, max_depth=8, seed=5, paths_per_pass=n)
        assert not got
        refs = [c.render_pt(sc.camera, k, max_depth=8, seed=5, paths_per_pass=n)[0] for k in (1, 2, 3)]
        vrefs = [c.render_vcm(sc.camera, k, 0.1, max_depth=8, seed=3)[0] for k in (1, 2, 3)]
    assert [s for _, s, _ in pt] == [1.0, 2.0, 3.0] and [s for _, s, _ in vcm] == [1.0, 2.0, 3.0]
    for snaps in (pt, vcm):
        ts = [t for t, _, _ in snaps]
        assert ts == sorted(ts) and ts[0] > 0
    for (_, _, img), ref in zip(pt, refs):
        assert np.allclose(img, ref, rtol=1e-9, atol=1e-12)
    for (_, _, img), ref in zip(vcm, vrefs):
        np.testing.assert_allclose(img, ref, rtol=1e-5, atol=1e-6 * ref.max())
