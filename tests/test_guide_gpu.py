"""GPU checks of the guiding network's tensor-core kernels against the FP64 oracle
(oracle/guide_mlp.py): the tcgen05 operand layouts, the forward pass, the training
kernel's gradient, and that Adam steps on the GPU reduce the loss."""
import itertools

import numpy as np
import pytest

import renderx_gb300 as rx
from oracle import guide_mlp as gm

pytestmark = pytest.mark.gpu
BOX = ((0.0, 0.0, 0.0), (5.56, 5.56, 5.56))


def bf16_bits(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def random_records(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 16), np.float32)
    r[:, 0:3] = rng.random((n, 3)) * 5.56
    for k in (3, 6, 9):
        v = rng.normal(size=(n, 3))
        r[:, k:k + 3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    r[:, 12] = rng.exponential(1.0, n)
    return r


@pytest.mark.parametrize("a_mn,b_mn", list(itertools.product([0, 1], [0, 1])))
@pytest.mark.parametrize("N,K", [(16, 16), (64, 64), (80, 128), (128, 80)])
def test_umma_m128_layouts_exact(a_mn, b_mn, N, K):
    rng = np.random.default_rng(N * 1000 + K + 10 * a_mn + b_mn)
    a = rng.integers(-2, 3, (128, K)).astype(np.float32)
    b = rng.integers(-2, 3, (N, K)).astype(np.float32)
    with rx.Context(0) as ctx:
        d = ctx.diag_umma_gemm(bf16_bits(a), bf16_bits(b), a_mn, b_mn)
    assert np.array_equal(d, a @ b.T)


@pytest.mark.parametrize("a_mn,b_mn", [(0, 0), (1, 1)])
@pytest.mark.parametrize("N", [64, 80])
def test_umma_m64_lane_placement(a_mn, b_mn, N):
    """An M = 64 accumulator occupies lanes 0..15 of each 32-lane quarter (row r in
    lane 32 (r // 16) + r % 16), the placement the training kernel's flush assumes."""
    rng = np.random.default_rng(N + 7 * a_mn)
    a = rng.integers(-2, 3, (64, 128)).astype(np.float32)
    b = rng.integers(-2, 3, (N, 128)).astype(np.float32)
    with rx.Context(0) as ctx:
        d = ctx.diag_umma_gemm(bf16_bits(a), bf16_bits(b), a_mn, b_mn)
    lanes = np.array([32 * (r // 16) + r % 16 for r in range(64)])
    assert np.array_equal(d[lanes], a @ b.T)


def test_forward_matches_oracle():
    recs = random_records(1000, 1)
    with rx.Context(0) as ctx:
        ctx.guide_init(seed=5, box=BOX)
        params = ctx.guide_params()
        raw, pdf = ctx.guide_eval(recs)
    assert np.array_equal(params, gm.init_params(5))
    _, ref = gm.forward(params, recs, *BOX)
    scale = np.abs(ref).max()
    err = np.abs(raw - ref).max() / scale
    assert err < 2e-2, err
    ref_pdf = gm.mixture_pdf(raw.astype(np.float64), recs[:, 9:12])
    assert np.allclose(pdf, ref_pdf, rtol=1e-3, atol=1e-6)


def test_gradient_matches_oracle():
    rng = np.random.default_rng(2)
    recs = random_records(4096 + 77, 3)  # ragged last tile
    with rx.Context(0) as ctx:
        ctx.guide_init(seed=9, box=BOX)
        p = gm.init_params(9)
        p = (p + rng.normal(scale=0.03, size=p.shape).astype(np.float32) * (p != 0)).astype(np.float32)
        ctx.guide_set_params(p)
        loss, g = ctx.guide_gradient(recs)
    ref_loss, ref = gm.gradient(p, recs, *BOX)
    assert abs(loss - ref_loss) <= 2e-3 * abs(ref_loss) + 1e-6
    for l in range(5):
        a, b = gm.W_OFF[l], gm.W_OFF[l] + 64 * gm.K_IN[l]
        rel = np.linalg.norm(g[a:b] - ref[a:b]) / max(np.linalg.norm(ref[a:b]), 1e-30)
        assert rel < 2e-2, (l, rel)
    last = g[gm.W_OFF[4]:].reshape(64, 64)
    assert np.all(last[40:] == 0)


def test_adam_steps_reduce_loss():
    """Records whose incident directions cluster about a position-dependent mean: a
    few hundred Adam steps on the GPU must lower the loss well below its start."""
    import torch
    rng = np.random.default_rng(4)
    n = 1 << 16
    recs = random_records(n, 8)
    mean = np.stack([np.cos(recs[:, 0]), np.sin(recs[:, 0]), 0.3 * np.ones(n)], 1)
    mean /= np.linalg.norm(mean, axis=1, keepdims=True)
    wi = mean + 0.15 * rng.normal(size=(n, 3))
    recs[:, 9:12] = wi / np.linalg.norm(wi, axis=1, keepdims=True)
    recs[:, 12] = 1.0
    d = torch.from_numpy(recs).cuda()
    with rx.Context(0) as ctx:
        ctx.guide_init(seed=1, box=BOX, learning_rate=5e-3, batch=n)
        first = ctx.guide_train_step(d.data_ptr(), n)
        for _ in range(300):
            last = ctx.guide_train_step(d.data_ptr(), n, want_loss=False)
        last = ctx.guide_train_step(d.data_ptr(), n)
    # uniform density on the sphere: -log(1/4pi) = 2.53; the fit to a lobe of spread
    # 0.15 rad (about 1.9 nats when matched exactly) is far lower
    assert 1.5 < first < 4.0 and last < first - 1.5, (first, last)


def _relmse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def test_guided_render_is_unbiased():
    """Guided sampling (network trained during the first passes of the same render, after
    BSDF-only warm-up passes) keeps the estimator's expectation: per pixel it agrees
    with a high-sample plain render within 3 sigma (at most 1% of channels, none beyond
    8), and its image mean agrees with the reference's own PathTracer render of the
    Cornell box within 4 standard errors."""
    from test_render_gpu import load_case
    z, sc = load_case("cornell_pt")
    spp = 8192
    with rx.Context(0) as ctx:
        ctx.set_scene(sc)
        ctx.build_accel()
        ref, ref_sq, _ = ctx.render_pt(sc.camera, 131072, max_depth=8, rr_mode=0, seed=1, want_sq=True)
        ctx.guide_init(seed=3, batch=1 << 16, warmup_passes=4, train_passes=8, steps_per_pass=8)
        mean, sq, st = ctx.render_pt(sc.camera, spp, max_depth=8, rr_mode=0, seed=777, want_sq=True, guided=True,
                                     paths_per_pass=1 << 18)
    se = np.sqrt(np.maximum(sq - mean * mean, 0.0) / (spp - 1))
    rse = np.sqrt(np.maximum(ref_sq - ref * ref, 0.0) / (131072 - 1))
    zz = np.abs(mean - ref) / (np.sqrt(se ** 2 + rse ** 2) + 1e-12)
    assert (zz > 3).mean() <= 0.01, f"{(zz > 3).mean():.4f} of channels beyond 3 sigma (max z {zz.max():.1f})"
    assert (zz > 8).sum() == 0
    gold, gse = z["mean"].astype(np.float64), z["stderr"].astype(np.float64)
    n = mean.shape[0] * mean.shape[1]
    for c in range(3):
        dm = mean[..., c].mean() - gold[..., c].mean()
        s_img = np.sqrt((se[..., c] ** 2).sum() + (gse[..., c] ** 2).sum()) / n
        assert abs(dm) < 4 * s_img, (c, dm, s_img)


def test_guided_render_is_unbiased_on_glossy_workload():
    """The workload guiding is for (glossy spheres with Phong exponents in [100, 1000], a
    light of 1% of the ceiling, Russian roulette from depth 3): a guided render, its
    network trained during the first passes of the same render, agrees per pixel with a
    plain BSDF-sampling render of 8x the samples within 3 sigma of the combined standard
    error (at most 1% of channels, none beyond 8; image means within 4 standard errors).
    One-sample MIS keeps the mixture density in the estimator's denominator, so any
    network, trained or not, leaves the expectation unchanged."""
    from renderx_gb300 import scenes
    sc = scenes.guiding_scene(64, 64, n_spheres=40, subdiv=3, seed=2)
    spp, ref_spp = 8192, 65536
    with rx.Context(0) as ctx:
        ctx.set_scene(sc)
        ctx.build_accel()
        ref, ref_sq, _ = ctx.render_pt(sc.camera, ref_spp, max_depth=8, rr_mode=1, seed=11, want_sq=True)
        ctx.guide_init(seed=4, batch=1 << 16, warmup_passes=4, train_passes=12, steps_per_pass=8)
        mean, sq, _ = ctx.render_pt(sc.camera, spp, max_depth=8, rr_mode=1, seed=12, want_sq=True, guided=True,
                                    paths_per_pass=1 << 17)
    se = np.sqrt(np.maximum(sq - mean * mean, 0.0) / (spp - 1))
    rse = np.sqrt(np.maximum(ref_sq - ref * ref, 0.0) / (ref_spp - 1))
    sig = np.sqrt(se ** 2 + rse ** 2)
    zz = np.abs(mean - ref) / (sig + 1e-12)
    bad = np.abs(mean - ref) > 3 * sig + 1e-4
    assert bad.mean() <= 0.01, f"{bad.mean():.4f} of channels beyond 3 sigma (max z {zz.max():.1f})"
    assert (zz > 8).sum() == 0, f"max z {zz.max():.1f}"
    n = mean.shape[0] * mean.shape[1]
    for c in range(3):
        dm = mean[..., c].mean() - ref[..., c].mean()
        s_img = np.sqrt((se[..., c] ** 2).sum() + (rse[..., c] ** 2).sum()) / n
        assert abs(dm) < 4 * s_img, (c, dm, s_img)


def test_guiding_gain_on_glossy_workload():
    """Equal-sample comparison on the glossy workload (60% glossy spheres, light of 1% of
    the ceiling): the guided path tracer, training and inference time included, needs
    well under the render time of plain BSDF sampling for the same relMSE against a
    high-sample FP64 reference (relMSE x time, which is constant for an unbiased
    estimator at a fixed sampler, below 0.6 of plain's)."""
    from renderx_gb300 import scenes
    sc = scenes.guiding_scene(128, 128, n_spheres=40, subdiv=3, seed=2)
    with rx.Context(0) as ctx:
        ctx.set_scene(sc)
        ctx.build_accel()
        ref, _, _ = ctx.render_pt(sc.camera, 32768, max_depth=8, rr_mode=1, seed=1)
        spp = 1024
        plain, _, sp = ctx.render_pt(sc.camera, spp, max_depth=8, rr_mode=1, seed=5, paths_per_pass=1 << 18)
        ctx.guide_init(seed=1, batch=1 << 16, warmup_passes=4, train_passes=12, steps_per_pass=8)
        guided, _, sg = ctx.render_pt(sc.camera, spp, max_depth=8, rr_mode=1, seed=6, guided=True,
                                      paths_per_pass=1 << 18)
    e_plain = _relmse(plain, ref) * sp["ms"]
    e_guided = _relmse(guided, ref) * sg["ms"]
    print(f"relMSE x ms: plain {e_plain:.4g} ({sp['ms']:.1f} ms), guided {e_guided:.4g} ({sg['ms']:.1f} ms)")
    assert e_guided < 0.6 * e_plain, (e_guided, e_plain)


def test_tensor_core_issue_rate_is_measured():
    """rx_diag_umma_rate: back-to-back BF16 MMAs (M = 128, K = 16) from one thread. The
    cycles per MMA grow with N and stay within the tensor core's bounds: an MMA of
    N = 256 (524,288 multiply-adds) cannot take less than 64 cycles on a core of at most
    8,192 multiply-adds per cycle, and none of the shapes takes 2,000."""
    with rx.Context(0) as ctx:
        rates = {n: ctx.diag_umma_rate(n, 256) for n in (64, 128, 256)}
    for n, (issue, done) in rates.items():
        assert 0 < issue <= done < 2000, (n, issue, done)
    assert rates[64][1] <= rates[256][1] and rates[256][1] >= 64

