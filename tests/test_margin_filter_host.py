"""The visibility check's margin filter (box_clear_pass in renderx_gb300/csrc/rx_exact.cuh)
must never call a box passed that the reference's box test rejects
(KDTree::Node::BoundingBox::intersect, reference src/KDTree.cpp:34-52): a wrong pass
would accept a winner the reference cannot see. Both are restated here in float32 (NumPy
rounds every single-precision operation to nearest, as the reference built without
fused multiply-adds does) and run over rays aimed within a few ulps of box edges and
corners, from origins inside and outside, at coordinates up to 10^3. The filter's face
point may be formed with or without a fused multiply-add on the GPU; both are checked.
The filter must also decide most rays that are not near an edge (else it saves nothing).
"""
import numpy as np

F = np.float32


def ref_box_pass(mn, mx, o, d):
    """The reference's box test, reduced to pass/fail: some face at a non-negative
    distance whose intersection point lies within the other two slabs, inclusive."""
    n = len(o)
    ok = np.zeros(n, bool)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        for i in range(6):
            a, a1, a2 = i % 3, (i + 1) % 3, (i + 2) % 3
            b = mn[:, a] if i < 3 else mx[:, a]
            da = d[:, a]
            dist = (b - o[:, a]) / da
            p1 = o[:, a1] + dist * d[:, a1]
            p2 = o[:, a2] + dist * d[:, a2]
            inter = (da != 0) & (dist >= 0) & (mn[:, a1] <= p1) & (mx[:, a1] >= p1) & (mn[:, a2] <= p2) & (mx[:, a2] >= p2)
            ok |= inter
    return ok


def filter_pass(mn, mx, o, d, fused):
    """box_clear_pass: 1 = passes (sound), 0 = undecided."""
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        inv = np.where(np.abs(d) > F(1e-30), F(1) / d, np.copysign(F(1e30), d)).astype(F)
        t0 = ((mn - o) * inv).astype(F)
        t1 = ((mx - o) * inv).astype(F)
        near, far = np.minimum(t0, t1), np.maximum(t0, t1)
        te, tx = near.max(axis=1), far.min(axis=1)
        mo = (F(4e-6) * (F(1) + np.abs(o))).astype(F)
        md = (F(4e-6) * np.abs(d)).astype(F)
        out = np.zeros(len(o), bool)
        for t, planes in ((te, near), (tx, far)):
            axis = np.argmax(planes == t[:, None], axis=1)  # the first axis attaining t
            tt = t[:, None]
            if fused:  # o + t d rounded once
                p = (o.astype(np.float64) + tt.astype(np.float64) * d.astype(np.float64)).astype(F)
            else:
                p = (o + (tt * d).astype(F)).astype(F)
            m = (tt.astype(np.float64) * md + mo).astype(F)  # one fused multiply-add
            inside = (p >= (mn + m).astype(F)) & (p <= (mx - m).astype(F))
            inside |= np.arange(3)[None, :] == axis[:, None]
            out |= (t >= 0) & inside.all(axis=1)
    return out


def adversarial_cases(n, seed):
    """Boxes of widely varying size and position; each ray aimed at a point on a box
    edge or corner moved by a few ulps, from an origin outside or inside the box."""
    rng = np.random.default_rng(seed)
    scale = 10.0 ** rng.uniform(-1, 3, n)
    lo = rng.uniform(-1, 1, (n, 3)) * scale[:, None]
    size = 10.0 ** rng.uniform(-3, 1, (n, 3)) * scale[:, None]
    mn, mx = lo.astype(F), (lo + size).astype(F)
    # a target on an edge or a corner: two or three coordinates on a face plane
    u = rng.uniform(0, 1, (n, 3))
    target = mn + (mx - mn) * u
    for k in range(3):
        snap = rng.random(n) < 0.7
        side = rng.random(n) < 0.5
        target[:, k] = np.where(snap, np.where(side, mn[:, k], mx[:, k]), target[:, k])
    target = target.astype(F)
    ulps = rng.integers(-4, 5, (n, 3))  # move each coordinate by up to four ulps
    toward = np.where(ulps > 0, np.inf, -np.inf).astype(F)
    for step in range(1, 5):
        target = np.where(np.abs(ulps) >= step, np.nextafter(target, toward), target).astype(F)
    inside = rng.random(n) < 0.3
    centre = ((mn.astype(np.float64) + mx) / 2)
    far = centre + rng.normal(size=(n, 3)) * (size + scale[:, None]) * 3
    near = mn + (mx - mn) * rng.uniform(0.05, 0.95, (n, 3))
    o = np.where(inside[:, None], near, far).astype(F)
    d = (target.astype(np.float64) - o).astype(np.float64)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(F)
    keep = np.all(d != 0, axis=1)  # zero components go to the exact test in the kernels
    return mn[keep], mx[keep], o[keep], d[keep]


def test_margin_filter_never_passes_a_box_the_reference_rejects():
    total = 0
    for seed in range(4):
        mn, mx, o, d = adversarial_cases(500_000, seed)
        ref = ref_box_pass(mn, mx, o, d)
        for fused in (False, True):
            got = filter_pass(mn, mx, o, d, fused)
            bad = np.nonzero(got & ~ref)[0]
            assert bad.size == 0, f"seed {seed} fused {fused}: {bad.size} unsound passes, first {bad[:3]}"
        total += len(o)
    assert total > 1_900_000


def test_margin_filter_decides_rays_away_from_edges():
    rng = np.random.default_rng(9)
    n = 200_000
    mn = rng.uniform(-5, 5, (n, 3)).astype(F)
    mx = (mn + rng.uniform(0.1, 3, (n, 3))).astype(F)
    o = rng.uniform(-20, 20, (n, 3)).astype(F)
    target = (mn + (mx - mn) * rng.uniform(0.2, 0.8, (n, 3))).astype(F)  # through the box's middle
    d = (target - o).astype(np.float64)
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(F)
    ref = ref_box_pass(mn, mx, o, d)
    got = filter_pass(mn, mx, o, d, True)
    assert ref.all()
    assert not (got & ~ref).any()
    assert got.mean() > 0.95
