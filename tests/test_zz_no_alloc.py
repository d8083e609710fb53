"""The allocation-free closest-hit entry point (rx_trace_closest_noalloc), called
through the C ABI, must return exactly what the allocating entry point
(rx_trace_closest_device) returns, on two calls in a row that share its fixed device
scratch array. It exists for callers that cannot allocate device memory while they
trace: hosts whose device memory belongs to their own pool allocator, or
latency-sensitive loops that must not pay cudaMalloc's implicit synchronisation.
Covered: every walk variant and both visibility-check kernels, and a batch with rays
whose closest triangle the reference's box tests hide (they go through the re-walk
queue, the second half of the scratch array). Collected last (file name), so a failure
here never hides the other tests."""
import numpy as np
import pytest

import oracle
import renderx_gb300 as rx
from renderx_gb300 import _capi, scenes
from golden_util import load

pytestmark = pytest.mark.gpu


def _noalloc(ctx, rays, n, tid, dist, stream):
    st = _capi.lib().rx_trace_closest_noalloc(ctx.h, _capi.ptr(rays), n, _capi.ptr(tid), _capi.ptr(dist),
                                              _capi.stream_arg(stream))
    _capi.check(ctx.h, st)


def _compare(ctx, torch, o, d):
    rays = torch.from_numpy(rx.rays_to_array(o, d)).cuda()
    n = rays.shape[0]
    stream = torch.cuda.current_stream().cuda_stream
    want_t = torch.empty(n, dtype=torch.int32, device="cuda")
    want_d = torch.empty(n, dtype=torch.float32, device="cuda")
    ctx.trace_closest_device(rays, n, want_t, want_d, stream)
    got_t = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    got_d = torch.full((n,), -7.0, dtype=torch.float32, device="cuda")
    _noalloc(ctx, rays, n, got_t, got_d, stream)
    torch.cuda.synchronize()
    assert torch.equal(got_t, want_t)
    assert torch.equal(got_d.view(torch.int32), want_d.view(torch.int32))  # bit-exact
    return got_t.cpu().numpy()


@pytest.mark.parametrize("variant", [0, 1, 3, 4, 5])
@pytest.mark.parametrize("check", [0, 1])
def test_noalloc_matches_allocating_entry_point_on_two_calls(variant, check):
    torch = pytest.importorskip("torch")
    z = load("spheres4")
    with rx.Context(0) as ctx:
        ctx.set_trace_config(variant, 4)
        ctx.set_trace_options(check, 1 << 18, 0)
        ctx.set_geometry(z["verts"], z["tris"])
        ctx.build_accel()
        o1, d1 = scenes.hit_rays(300_000, seed=31)
        o2, d2 = np.asarray(z["origins"]), np.asarray(z["dirs"])
        _compare(ctx, torch, o1, d1)  # two calls in a row, different batch sizes
        got = _compare(ctx, torch, o2, d2)
        # the golden batch also matches the reference's own answers
        assert np.array_equal(got, z["tid"])


def test_noalloc_rewalk_queue_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    z = load("cornell")
    T = oracle.RefTree(z["verts"], z["tris"])
    ut, ud = T.trace_unboxed(z["origins"], z["dirs"])
    hidden = (ut != z["tid"]) | (ud.view(np.int32) != np.asarray(z["dist"], np.float32).view(np.int32))
    assert hidden.sum() > 0  # rays that need the exact re-walk
    with rx.Context(0) as ctx:
        ctx.set_geometry(z["verts"], z["tris"])
        ctx.build_accel()
        ctx.counters(reset=True)
        for _ in range(2):
            got = _compare(ctx, torch, z["origins"], z["dirs"])
            assert np.array_equal(got, z["tid"])
        assert ctx.counters()["eager_retraces"] >= 2 * int(hidden.sum())  # the allocating calls re-walked them


def test_noalloc_rejects_batches_beyond_its_limit():
    torch = pytest.importorskip("torch")
    z = load("cornell")
    with rx.Context(0) as ctx:
        ctx.set_geometry(z["verts"], z["tris"])
        ctx.build_accel()
        n = (1 << 20) + 1
        rays = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
        tid = torch.empty(n, dtype=torch.int32, device="cuda")
        dist = torch.empty(n, dtype=torch.float32, device="cuda")
        with pytest.raises(rx.RxError, match="exceed the limit of 1048576"):
            _noalloc(ctx, rays, n, tid, dist, None)
