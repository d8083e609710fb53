"""CPU checks of the guiding network's FP64 restatement (oracle/guide_mlp.py): its
analytic gradient against central finite differences, the mixture density's
normalisation, and the BF16 rounding helper."""
import numpy as np
import pytest

from oracle import guide_mlp as gm


def random_records(n, seed, box=((0, 0, 0), (5.56, 5.56, 5.56))):
    rng = np.random.default_rng(seed)
    mn, mx = np.array(box[0], float), np.array(box[1], float)
    r = np.zeros((n, 16), np.float32)
    r[:, 0:3] = mn + rng.random((n, 3)) * (mx - mn)
    for k in (3, 6, 9):
        v = rng.normal(size=(n, 3))
        r[:, k:k + 3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    r[:, 12] = rng.exponential(1.0, n)
    return r


def test_bf16_round_ties_to_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0, 1e-30], np.float32)
    got = gm.bf16_round(x)
    assert got[0] == 1.0
    assert got[1] == 1.0                     # tie -> even mantissa
    assert got[2] == 1.0 + 4 * 2 ** -8       # tie -> even (up)
    assert got[3] == -2.5 and got[4] == 0.0
    assert abs(got[5] - 1e-30) / 1e-30 < 2 ** -8


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    params = gm.init_params(11).astype(np.float64)
    params += rng.normal(scale=0.05, size=params.shape) * (params != 0)  # move off the init
    recs = random_records(24, 5)
    box = ((0, 0, 0), (5.56, 5.56, 5.56))
    loss, g = gm.gradient(params, recs, *box, emulate_bf16=False)
    idx = np.concatenate([rng.choice(np.arange(l0, l0 + 64 * k), 8, replace=False)
                          for l0, k in zip(gm.W_OFF, gm.K_IN)])
    idx = idx[np.abs(params[idx]) > 0] if (np.abs(params[idx]) > 0).any() else idx
    h = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += h
        p2[i] -= h
        l1, _ = gm.gradient(p1, recs, *box, emulate_bf16=False)
        l2, _ = gm.gradient(p2, recs, *box, emulate_bf16=False)
        fd = (l1 - l2) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 + 1e-4 * abs(fd), (i, fd, g[i])
    assert np.isfinite(loss)


def test_mixture_density_integrates_to_one():
    rng = np.random.default_rng(1)
    raw = rng.normal(size=(1, 40))
    raw[0, 1::5] = rng.uniform(-2, 4, 8)  # kappa in [0.14, 55]
    # quadrature over the sphere: uniform directions
    n = 400000
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    pdf = gm.mixture_pdf(np.repeat(raw, n, axis=0), v)
    est = pdf.mean() * 4 * np.pi
    assert abs(est - 1.0) < 0.03, est


def test_init_params_layout():
    w = gm.init_params(7)
    assert w.shape == (gm.N_PARAMS,)
    last = w[gm.W_OFF[4]:].reshape(64, 64)
    assert np.all(last[40:] == 0) and np.any(last[:40] != 0)
    first = w[:5120]
    a = np.sqrt(6.0 / 80)
    assert np.abs(first).max() <= a and np.abs(first).max() > 0.9 * a


@pytest.mark.parametrize("emulate", [True, False])
def test_forward_shapes_and_scale(emulate):
    recs = random_records(32, 9)
    acts, raw = gm.forward(gm.init_params(3), recs, (0, 0, 0), (5.56, 5.56, 5.56), emulate)
    assert raw.shape == (32, 40) and len(acts) == 5
    assert np.isfinite(raw).all()
    pdf = gm.mixture_pdf(raw, recs[:, 9:12])
    assert (pdf > 0).all()
