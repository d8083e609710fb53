"""ORACLE — test infrastructure only.

FP64 CPU restatement of the path-guiding network (no reference counterpart: the
network is this project's learned proposal). It mirrors the GPU kernels' arithmetic
contract: BF16 weights, BF16 inputs and hidden activations, BF16 back-propagated
pre-activation gradients, everything else exact (FP64 here, FP32 accumulation on the
GPU), so the two agree to the rounding of an occasional BF16 value. With
``emulate_bf16=False`` every rounding step is skipped, which gives the exact gradient
the finite-difference test checks.

Records are (n, 16) float32: position, shading normal, outgoing direction, incident
direction, weight, 3 unused. The network: 80 inputs -> 4 x 64 ReLU -> 64 outputs of
which 40 are 8 lobes x (weight logit, log-concentration, mean xyz).
"""
from __future__ import annotations

import numpy as np

K_IN = (80, 64, 64, 64, 64)
W_OFF = (0, 5120, 9216, 13312, 17408)
N_PARAMS = 21504
LOBES = 8
LOGK_MIN, LOGK_MAX = -4.0, 8.0


def bf16_round(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layers(params: np.ndarray, emulate_bf16: bool = True) -> list[np.ndarray]:
    """Per-layer weight matrices [64][K] (BF16-rounded as the kernels see them)."""
    out = []
    for l in range(5):
        w = np.asarray(params[W_OFF[l]:W_OFF[l] + 64 * K_IN[l]], np.float64).reshape(64, K_IN[l])
        out.append(bf16_round(w) if emulate_bf16 else w)
    return out


def encode(recs: np.ndarray, box_min, box_max) -> np.ndarray:
    """(n, 80) inputs: sin/cos(pi 2^f p_c) for c < 3, f < 12 (feature c*24 + 2f + {0,1}),
    normal, outgoing direction, 1, 0; p_c = (x_c - min_c) / extent_c in float32."""
    r = np.asarray(recs, np.float32)
    mn = np.asarray(box_min, np.float32)
    ext = (np.asarray(box_max, np.float32) - mn).astype(np.float32)
    p = ((r[:, 0:3] - mn).astype(np.float32) / ext).astype(np.float32).astype(np.float64)
    n = len(r)
    x = np.zeros((n, 80))
    for c in range(3):
        for f in range(12):
            a = np.pi * (2.0 ** f) * p[:, c]
            x[:, c * 24 + 2 * f] = np.sin(a)
            x[:, c * 24 + 2 * f + 1] = np.cos(a)
    x[:, 72:75] = r[:, 3:6]
    x[:, 75:78] = r[:, 6:9]
    x[:, 78] = 1.0
    return x


def forward(params, recs, box_min, box_max, emulate_bf16: bool = True):
    """Returns (activations [A0..A4], raw outputs (n, 40))."""
    Ws = layers(params, emulate_bf16)
    rnd = bf16_round if emulate_bf16 else (lambda v: np.asarray(v, np.float64))
    a = rnd(encode(recs, box_min, box_max))
    acts = [a]
    for l in range(4):
        a = rnd(np.maximum(a @ Ws[l].T, 0.0))
        acts.append(a)
    raw = acts[4] @ Ws[4].T
    return acts, raw[:, :40]


def decode(raw):
    """Mixture parameters: log weights, kappa, in-range mask, means, mean lengths, log
    vMF normalisers."""
    raw = np.asarray(raw, np.float64).reshape(-1, LOBES, 5)
    a = raw[..., 0]
    logpi = a - (a.max(1, keepdims=True) + np.log(np.exp(a - a.max(1, keepdims=True)).sum(1, keepdims=True)))
    b = raw[..., 1]
    kin = (b > LOGK_MIN) & (b < LOGK_MAX)
    kappa = np.exp(np.clip(b, LOGK_MIN, LOGK_MAX))
    m = raw[..., 2:5]
    ln = np.maximum(np.linalg.norm(m, axis=-1), 1e-6)
    mu = m / ln[..., None]
    lognorm = np.log(kappa) - np.log(2 * np.pi) - np.log(-np.expm1(-2 * kappa))
    return logpi, kappa, kin, mu, ln, lognorm


def mixture_pdf(raw, wi) -> np.ndarray:
    logpi, kappa, _, mu, _, lognorm = decode(raw)
    t = np.einsum("njk,nk->nj", mu, np.asarray(wi, np.float64))
    return np.exp(logpi + lognorm + kappa * (t - 1.0)).sum(1)


def loss_grad(raw, wi, scale):
    """Per-sample -scale log q(wi) and its gradient with respect to the raw outputs."""
    logpi, kappa, kin, mu, ln, lognorm = decode(raw)
    wi = np.asarray(wi, np.float64)
    t = np.einsum("njk,nk->nj", mu, wi)
    lv = logpi + lognorm + kappa * (t - 1.0)
    mx = lv.max(1, keepdims=True)
    lq = mx[:, 0] + np.log(np.exp(lv - mx).sum(1))
    g = np.exp(lv - lq[:, None])
    s = np.asarray(scale, np.float64)[:, None]
    d = np.zeros((len(lq), LOBES, 5))
    d[..., 0] = s * (np.exp(logpi) - g)
    with np.errstate(over="ignore"):
        dk = 1.0 - 2.0 * kappa / np.expm1(2.0 * kappa) + kappa * (t - 1.0)
    d[..., 1] = np.where(kin, -s * g * dk, 0.0)
    c = -s * g * kappa / ln
    d[..., 2:5] = c[..., None] * (wi[:, None, :] - t[..., None] * mu)
    return -s[:, 0] * lq, d.reshape(-1, 40)


def batch_scale(recs) -> np.ndarray:
    """Per-record loss weight: weight clipped at 32 x the batch mean, over the batch sum."""
    w = np.asarray(recs, np.float32)[:, 12].astype(np.float64)
    total = np.float32(w.sum())
    clip = np.float32(32.0) * total / np.float32(max(len(w), 1))
    return np.minimum(w, clip) / total if total > 0 else np.zeros_like(w)


def gradient(params, recs, box_min, box_max, emulate_bf16: bool = True):
    """Batch loss and its gradient with respect to the 21504 parameters."""
    rnd = bf16_round if emulate_bf16 else (lambda v: np.asarray(v, np.float64))
    Ws = layers(params, emulate_bf16)
    acts, raw = forward(params, recs, box_min, box_max, emulate_bf16)
    wi = np.asarray(recs, np.float32)[:, 9:12]
    loss, dz = loss_grad(raw, wi, batch_scale(recs))
    dzf = np.zeros((len(dz), 64))
    dzf[:, :40] = dz
    dz = rnd(dzf)
    grad = np.zeros(N_PARAMS)
    for l in range(4, -1, -1):
        gw = dz.T @ acts[l]
        grad[W_OFF[l]:W_OFF[l] + 64 * K_IN[l]] = gw.reshape(-1)
        if l > 0:
            da = dz @ Ws[l]
            dz = rnd(np.where(acts[l] > 0, da, 0.0))
    return float(loss.sum()), grad


def init_params(seed: int) -> np.ndarray:
    """Seeded initial parameters in the library's scheme (He-uniform, output layer x0.1,
    unused output rows zero): splitmix64 of (seed, index) -> uniform [-1, 1)."""
    M = (1 << 64) - 1
    w = np.zeros(N_PARAMS, np.float32)
    for l in range(5):
        k = K_IN[l]
        a = np.float32(np.sqrt(np.float32(6.0) / np.float32(k))) * (np.float32(0.1) if l == 4 else np.float32(1.0))
        rows = 40 if l == 4 else 64
        for r in range(rows):
            for c in range(k):
                i = W_OFF[l] + r * k + c
                z = (seed + 0x9E3779B97F4A7C15 * (i + 1)) & M
                z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
                z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
                z ^= z >> 31
                u = np.float32((z >> 40) * (1.0 / 16777216.0)) * np.float32(2.0) - np.float32(1.0)
                w[i] = a * u
    return w
