"""GPU closest-hit parity: the sm_103a kernels, called through the C ABI, return the
reference's answers bit for bit (triangle ids and distances), against the golden
fixtures made by the reference's own KDTree and against the oracle restatement."""
import numpy as np
import pytest

import oracle
import renderx_gb300 as rx
from renderx_gb300 import scenes
from golden_util import CASES, load

pytestmark = pytest.mark.gpu


def _bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.int32), np.asarray(b, np.float32).view(np.int32))


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("leaf_size", [1, 3, 4, 8])
@pytest.mark.parametrize("variant", [0, 1, 3, 4, 5])
@pytest.mark.parametrize("check", [0, 1])
def test_hits_match_reference_golden(name, leaf_size, variant, check):
    z = load(name)
    with rx.Context(0) as ctx:
        ctx.set_trace_config(variant, 4)
        # bin even the small golden batches; both walk stack depths
        ctx.set_trace_options(check, 64 if check else 0, 32 if check else 64)
        ctx.set_geometry(z["verts"], z["tris"])
        ctx.build_accel(rx.SPLIT_GCC, leaf_size=leaf_size)
        tid, dist = ctx.trace_closest(z["origins"], z["dirs"])
        c = ctx.counters()
    bad = np.nonzero(tid != z["tid"])[0]
    assert bad.size == 0, f"{bad.size} id mismatches, first {bad[:5]}: got {tid[bad[:5]]} want {z['tid'][bad[:5]]}"
    assert _bits_equal(dist, z["dist"])
    assert c["errors"] == 0


@pytest.mark.parametrize("name", CASES)
def test_reference_order_walk_matches_golden(name):
    torch = pytest.importorskip("torch")
    z = load(name)
    with rx.Context(0) as ctx:
        ctx.set_geometry(z["verts"], z["tris"])
        ctx.build_accel()
        rays = torch.from_numpy(rx.rays_to_array(z["origins"], z["dirs"])).cuda()
        n = rays.shape[0]
        tid = torch.empty(n, dtype=torch.int32, device="cuda")
        dist = torch.empty(n, dtype=torch.float32, device="cuda")
        ctx.trace_reforder_device(rays, n, tid, dist)
        torch.cuda.synchronize()
        assert np.array_equal(tid.cpu().numpy(), z["tid"])
        assert _bits_equal(dist.cpu().numpy(), z["dist"])
        # device-buffer entry point of the fast path, on torch's stream
        tid2 = torch.empty_like(tid)
        dist2 = torch.empty_like(dist)
        ctx.trace_closest_device(rays, n, tid2, dist2, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert np.array_equal(tid2.cpu().numpy(), z["tid"])
        assert _bits_equal(dist2.cpu().numpy(), z["dist"])


def test_best_axis_policy_matches_oracle():
    z = load("spheres4")
    T = oracle.RefTree(z["verts"], z["tris"], oracle.SPLIT_BEST)
    want_t, want_d = T.trace(z["origins"], z["dirs"])
    with rx.Context(0) as ctx:
        ctx.set_geometry(z["verts"], z["tris"])
        ctx.build_accel(rx.SPLIT_BEST)
        tid, dist = ctx.trace_closest(z["origins"], z["dirs"])
    assert np.array_equal(tid, want_t)
    assert _bits_equal(dist, want_d)


def test_empty_and_single_triangle_and_ragged_batches():
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    t = np.array([[0, 1, 2]], np.uint32)
    with rx.Context(0) as ctx:
        ctx.set_geometry(v, t)
        ctx.build_accel()
        tid, dist = ctx.trace_closest(np.zeros((0, 3)), np.zeros((0, 3)))
        assert tid.size == 0
        T = oracle.RefTree(v, t)
        for n in (1, 31, 33, 129, 1000):
            o, d = scenes.hit_rays(n, seed=n, lo=-0.5, hi=1.5)
            tid, dist = ctx.trace_closest(o, d)
            wt, wd = T.trace(o, d)
            assert np.array_equal(tid, wt) and _bits_equal(dist, wd)


def test_invalid_inputs_raise():
    with rx.Context(0) as ctx:
        with pytest.raises(rx.RxError):
            ctx.trace_closest(np.zeros((4, 3)), np.ones((4, 3)))  # before build
        v = np.zeros((3, 3), np.float32)
        with pytest.raises(rx.RxError):
            ctx.set_geometry(v, np.array([[0, 1, 3]], np.uint32))  # index out of range
        v[0, 0] = np.nan
        with pytest.raises(rx.RxError):
            ctx.set_geometry(v, np.array([[0, 1, 2]], np.uint32))
        for key in ((2, 2, 0), (6, 1, 0), (4, 4, 0), (5, 3, 0), (4, 5, 1), (3, 7, 1), (4, 2, 2)):  # out of range
            with pytest.raises(rx.RxError):
                ctx.set_trace_binning(*key)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("key", [(3, 1, 0), (3, 3, 0), (5, 2, 0), (4, 3, 0), (4, 4, 1), (3, 6, 1), (5, 1, 1)])
def test_binning_key_does_not_change_answers(name, key):
    """Every binning key the options allow orders the rays differently and returns the
    reference's answers bit for bit (the golden batches, binned from 64 rays on)."""
    z = load(name)
    with rx.Context(0) as ctx:
        ctx.set_trace_options(1, 64, 0)
        ctx.set_trace_binning(*key)
        ctx.set_geometry(z["verts"], z["tris"])
        ctx.build_accel()
        tid, dist = ctx.trace_closest(z["origins"], z["dirs"])
    assert np.array_equal(tid, z["tid"])
    assert _bits_equal(dist, z["dist"])


@pytest.mark.parametrize("stage,n", [(1 << 16, 5 * (1 << 16) + 77), (1 << 20, 3 * (1 << 20) + 12345)])
def test_host_buffer_ring_matches_device_path(stage, n):
    """The host-buffer call stages the rays through a three-slot ring (copies in on one
    stream, each slot's kernels on their own, copies out on another, ordered by events)
    in chunks that ramp up to the staging size: equal chunks of 2^16 (five and a ragged
    tail, each slot reused), and 2^18, 2^19, 2^20, 2^20 plus a tail. Every answer equals
    the device-buffer call's."""
    torch = pytest.importorskip("torch")
    sc = scenes.sphere_field(20, 3, seed=2)
    f = sc.flatten()
    o, d = scenes.hit_rays(n, seed=11)
    with rx.Context(0) as ctx:
        ctx.set_geometry(f["verts"], f["tris"])
        ctx.build_accel()
        rays = torch.from_numpy(rx.rays_to_array(o, d)).cuda()
        tid = torch.empty(n, dtype=torch.int32, device="cuda")
        dist = torch.empty(n, dtype=torch.float32, device="cuda")
        ctx.trace_closest_device(rays, n, tid, dist)
        torch.cuda.synchronize()
        ctx.set_trace_staging(stage)
        for _ in range(2):  # twice: the second call reuses the ring and its events
            ht, hd = ctx.trace_closest(o, d)
            assert np.array_equal(ht, tid.cpu().numpy())
            assert _bits_equal(hd, dist.cpu().numpy())
        assert ctx.counters()["errors"] == 0


@pytest.mark.slow
def test_full_size_batch_matches_oracle_sample_and_reference_walk():
    """4,096,036 triangles, 2^24 rays: the whole batch through the fast path; a sample
    against the CPU oracle; a stratified 2^21-ray sample (eight 2^18-ray windows spread
    evenly over the batch, one launch each) against the reference-order walk on the GPU,
    whose traversal is independent of the fast path's (it visits every node whose box
    passes, in the reference's order, with no BVH, no pruning and no visibility check, so
    it costs nearly a brute-force test per ray; only the exact box and triangle
    arithmetic, pinned to the goldens, is shared); the whole batch twice for determinism, through every walk
    variant and check mode, and once more from host buffers (staged chunks)."""
    torch = pytest.importorskip("torch")
    sc = scenes.sphere_field(200, 5, seed=1)
    f = sc.flatten()
    n = 1 << 24
    o, d = scenes.hit_rays(n, seed=7)
    with rx.Context(0) as ctx:
        ctx.set_geometry(f["verts"], f["tris"])
        ctx.build_accel()
        rays = torch.from_numpy(rx.rays_to_array(o, d)).cuda()
        tid = torch.empty(n, dtype=torch.int32, device="cuda")
        dist = torch.empty(n, dtype=torch.float32, device="cuda")
        ctx.trace_closest_device(rays, n, tid, dist)
        tid2, dist2 = torch.empty_like(tid), torch.empty_like(dist)
        ctx.trace_closest_device(rays, n, tid2, dist2)
        torch.cuda.synchronize()
        assert torch.equal(tid, tid2) and torch.equal(dist.view(torch.int32), dist2.view(torch.int32))
        for variant in (0, 1, 3, 5):  # every walk variant returns the same answers on the whole batch
            ctx.set_trace_config(variant, 12)
            ctx.trace_closest_device(rays, n, tid2, dist2)
            torch.cuda.synchronize()
            assert torch.equal(tid, tid2) and torch.equal(dist.view(torch.int32), dist2.view(torch.int32)), variant
        ctx.set_trace_config(4, 12)
        ctx.set_trace_options(0)  # the warp-per-ray check: the same answers as thread per ray
        ctx.trace_closest_device(rays, n, tid2, dist2)
        torch.cuda.synchronize()
        assert torch.equal(tid, tid2) and torch.equal(dist.view(torch.int32), dist2.view(torch.int32))
        ctx.set_trace_options(1)
        m = 1 << 18
        tr = torch.empty(m, dtype=torch.int32, device="cuda")
        dr = torch.empty(m, dtype=torch.float32, device="cuda")
        checked = 0
        for w in range(8):  # windows at 0, 2^21, 2 x 2^21, ...: every eighth of the batch
            a = w * (n // 8)
            ctx.trace_reforder_device(rays[a:a + m], m, tr, dr)
            torch.cuda.synchronize()
            assert torch.equal(tr, tid[a:a + m]), (w, int((tr != tid[a:a + m]).sum()))
            assert torch.equal(dr.view(torch.int32), dist[a:a + m].view(torch.int32)), w
            checked += m
        assert checked == 1 << 21
        ht, hd = ctx.trace_closest(o, d)
        assert ctx.counters()["errors"] == 0
    tid = tid.cpu().numpy()
    dist = dist.cpu().numpy()
    assert np.array_equal(ht, tid) and _bits_equal(hd, dist)
    rng = np.random.default_rng(0)
    sample = np.sort(rng.choice(n, 1024, replace=False))
    T = oracle.RefTree(f["verts"], f["tris"])
    wt, wd = T.trace(o[sample], d[sample])
    assert np.array_equal(tid[sample], wt)
    assert _bits_equal(dist[sample], wd)
    assert 0.5 < (tid >= 0).mean() <= 1.0
