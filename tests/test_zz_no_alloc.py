"""The allocation-free closest-hit entry point (rx_trace_closest_noalloc), called
through the C ABI, must return exactly what the allocating entry point
(rx_trace_closest_device) returns, on two calls in a row that share its fixed device
scratch array. It exists for callers that cannot allocate device memory while they
trace: hosts whose device memory belongs to their own pool allocator, or
latency-sensitive loops that must not pay cudaMalloc's implicit synchronisation.
Collected last (file name), so a failure here never hides the other tests."""
import ctypes

import numpy as np
import pytest

import renderx_gb300 as rx
from renderx_gb300 import _capi, scenes
from golden_util import load

pytestmark = pytest.mark.gpu


def _noalloc(ctx, rays, n, tid, dist, stream):
    st = _capi.lib().rx_trace_closest_noalloc(ctx.h, _capi.ptr(rays), n, _capi.ptr(tid), _capi.ptr(dist),
                                              _capi.stream_arg(stream))
    _capi.check(ctx.h, st)


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    z = load("spheres4")
    with rx.Context(0) as ctx:
        ctx.set_geometry(z["verts"], z["tris"])
        ctx.build_accel()
        o1, d1 = scenes.hit_rays(300_000, seed=31)
        o2, d2 = np.asarray(z["origins"]), np.asarray(z["dirs"])
        for o, d in ((o1, d1), (o2, d2)):  # two calls in a row, different batch sizes
            rays = torch.from_numpy(rx.rays_to_array(o, d)).cuda()
            n = rays.shape[0]
            want_t = torch.empty(n, dtype=torch.int32, device="cuda")
            want_d = torch.empty(n, dtype=torch.float32, device="cuda")
            ctx.trace_closest_device(rays, n, want_t, want_d, torch.cuda.current_stream().cuda_stream)
            got_t = torch.full((n,), -7, dtype=torch.int32, device="cuda")
            got_d = torch.full((n,), -7.0, dtype=torch.float32, device="cuda")
            _noalloc(ctx, rays, n, got_t, got_d, torch.cuda.current_stream().cuda_stream)
            torch.cuda.synchronize()
            assert torch.equal(got_t, want_t)
            assert torch.equal(got_d.view(torch.int32), want_d.view(torch.int32))  # bit-exact
        # the golden batch also matches the reference's own answers
        assert np.array_equal(got_t.cpu().numpy(), z["tid"])


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
