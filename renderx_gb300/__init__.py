"""renderx_gb300 — GB300-native (sm_103a) light-transport hot path of RenderX.

The compute lives in librenderx_gb300.so (CUDA kernels behind the C ABI of
include/renderx.h); this package is a thin host-side mirror of the reference's
interfaces for the path:

* :class:`KDTree` mirrors the reference's triangle KDTree (include/KDTree.h:10-59):
  ``vertexPositionList`` / ``triangleList``, ``build()``, ``intersect()`` (batched) and
  ``serializeForGPU()``.
* :class:`Context` is the C-ABI context: scene upload, accelerator build, closest-hit
  batches on host or device buffers.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import (RxError, rx_bpt_options, rx_build_options, rx_camera, rx_object, rx_pm_options, rx_pt_options,
                    rx_render_stats, rx_vcm_options)
from . import scenes

__all__ = ["Context", "KDTree", "RxError", "reftree_serialize", "scenes", "rays_to_array"]

SPLIT_GCC = 0
SPLIT_BEST = 1


def rays_to_array(origins: np.ndarray, dirs: np.ndarray) -> np.ndarray:
    """Packs rays into the ABI's 32-byte rx_ray records: (n, 8) float32."""
    o = np.asarray(origins, np.float32).reshape(-1, 3)
    d = np.asarray(dirs, np.float32).reshape(-1, 3)
    r = np.zeros((len(o), 8), np.float32)
    r[:, 0:3] = o
    r[:, 4:7] = d
    return r


def reftree_serialize(verts: np.ndarray, tris: np.ndarray, policy: int = SPLIT_GCC):
    """KDTree::serializeForGPU of the library's reference-order tree (host only)."""
    L = _capi.lib()
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(tris, np.uint32).reshape(-1, 3)
    nn, nl = ctypes.c_uint32(0), ctypes.c_uint32(0)
    _capi.check(None, L.rx_reftree_serialize(_capi.ptr(v), len(v), _capi.ptr(t), len(t), policy, None,
                                             ctypes.byref(nn), None, ctypes.byref(nl)))
    nodes = np.zeros((nn.value, 12), np.float32)
    leaf = np.zeros(nl.value, np.float32)
    _capi.check(None, L.rx_reftree_serialize(_capi.ptr(v), len(v), _capi.ptr(t), len(t), policy, _capi.ptr(nodes),
                                             ctypes.byref(nn), _capi.ptr(leaf), ctypes.byref(nl)))
    return nodes, leaf


def config_read(path: str) -> tuple[dict, dict]:
    """rx_config_read: the library's C++ reader of the reference's config / scene XML and
    meshes (host only). Returns (arrays: verts, tris, tri_obj, tri_local, normals or None,
    objects (list of rx_object), info dict)."""
    L = _capi.lib()
    h = ctypes.c_void_p()
    info = _capi.rx_config_info()
    err = ctypes.create_string_buffer(512)
    st = L.rx_config_read(path.encode(), ctypes.byref(h), ctypes.byref(info), err, len(err))
    if st != 0:
        raise RxError(st, err.value.decode())
    try:
        pv, pt, po, pl, pn, pob = (ctypes.c_void_p() for _ in range(6))
        nv, nt, nobj = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        _capi.check(None, L.rx_host_scene_arrays(h, ctypes.byref(pv), ctypes.byref(nv), ctypes.byref(pt),
                                                 ctypes.byref(nt), ctypes.byref(po), ctypes.byref(pl),
                                                 ctypes.byref(pn), ctypes.byref(pob), ctypes.byref(nobj)))

        def arr(p, n, ct, shape):
            if not p.value or n == 0:
                return np.zeros(shape, np.dtype(ct))
            buf = (ct * n).from_address(p.value)
            return np.ctypeslib.as_array(buf).reshape(shape).copy()
        out = dict(verts=arr(pv, 3 * nv.value, ctypes.c_float, (nv.value, 3)),
                   tris=arr(pt, 3 * nt.value, ctypes.c_uint32, (nt.value, 3)),
                   tri_obj=arr(po, nt.value, ctypes.c_uint32, (nt.value,)),
                   tri_local=arr(pl, nt.value, ctypes.c_uint32, (nt.value,)),
                   normals=arr(pn, 3 * nv.value, ctypes.c_float, (nv.value, 3)) if pn.value else None,
                   objects=[rx_object.from_buffer_copy((rx_object * nobj.value).from_address(pob.value)[k])
                            for k in range(nobj.value)])
    finally:
        L.rx_host_scene_free(h)
    c = info.camera
    meta = dict(renderer=info.renderer.decode(), estimator=info.estimator, max_depth=info.max_depth, spp=info.spp,
                radius=info.radius, runtime_s=info.runtime_s, num_objects=info.num_objects,
                num_triangles=info.num_triangles, save_path=info.save_path.decode(),
                camera=scenes.Camera(c.width, c.height, c.sight_dist, tuple(c.position), tuple(c.focus), tuple(c.up)))
    return out, meta


def write_pfm(path: str, rgb: np.ndarray):
    """rx_write_pfm: MCRenderer::saveImagePFM of an (H, W, 3) image (rows from the top)."""
    a = np.ascontiguousarray(rgb, np.float64)
    h, w, _ = a.shape
    _capi.check(None, _capi.lib().rx_write_pfm(path.encode(), w, h, _capi.ptr(a)))


class Context:
    """One device, one stream: rx_create / rx_destroy."""

    def __init__(self, device: int = 0):
        self._L = _capi.lib()
        h = ctypes.c_void_p()
        st = self._L.rx_create(ctypes.byref(h), device)
        if st != 0:
            raise RxError(st, f"rx_create(device={device}) failed")
        self.h = h
        self.num_triangles = 0

    def close(self):
        if getattr(self, "h", None):
            self._L.rx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, st):
        _capi.check(self.h, st)

    # -- scene ---------------------------------------------------------------------
    def set_geometry(self, verts, tris, tri_obj=None, tri_local=None, normals=None):
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(tris, np.uint32).reshape(-1, 3)
        to = None if tri_obj is None else np.ascontiguousarray(tri_obj, np.uint32)
        tl = None if tri_local is None else np.ascontiguousarray(tri_local, np.uint32)
        n = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        self._ck(self._L.rx_scene_set_geometry(self.h, _capi.ptr(v), len(v), _capi.ptr(t), len(t), _capi.ptr(to),
                                               _capi.ptr(tl), _capi.ptr(n)))
        self.num_triangles = len(t)

    def set_objects(self, objs):
        arr = (rx_object * max(1, len(objs)))(*objs)
        self._ck(self._L.rx_scene_set_objects(self.h, ctypes.cast(arr, ctypes.c_void_p), len(objs)))

    def load_config(self, path: str) -> dict:
        """rx_scene_load_config: the reference's config / scene XML and meshes straight
        into this context (then build_accel). Returns the config's renderer settings."""
        info = _capi.rx_config_info()
        self._ck(self._L.rx_scene_load_config(self.h, path.encode(), ctypes.byref(info)))
        c = info.camera
        return dict(renderer=info.renderer.decode(), estimator=info.estimator, max_depth=info.max_depth,
                    spp=info.spp, radius=info.radius, runtime_s=info.runtime_s,
                    camera=scenes.Camera(c.width, c.height, c.sight_dist, tuple(c.position), tuple(c.focus),
                                         tuple(c.up)))

    def set_scene(self, scene: "scenes.Scene"):
        """Uploads a scenes.Scene: geometry (object-major, as Scene::buildKDTree) and
        the per-object material table."""
        f = scene.flatten()
        self.set_geometry(f["verts"], f["tris"], f["tri_obj"], f["tri_local"], f["normals"])
        self.set_objects(objects_from_scene(scene))
        return f

    def build_accel(self, split_policy: int = SPLIT_GCC, leaf_size: int = 0, host_threads: int = 0):
        o = rx_build_options(split_policy, leaf_size, host_threads, 0)
        self._ck(self._L.rx_build_accel(self.h, ctypes.byref(o)))

    def stats(self) -> dict:
        out = np.zeros(8, np.int64)
        self._ck(self._L.rx_accel_stats(self.h, _capi.ptr(out)))
        return dict(bvh_nodes=int(out[0]), bvh_depth=int(out[1]), ref_nodes=int(out[2]), ref_depth=int(out[3]),
                    triangles=int(out[4]), ref_leaves=int(out[5]), bvh4_depth=int(out[6]),
                    bvh8_depth=int(out[7]))

    # -- closest hit -----------------------------------------------------------------
    def trace_closest(self, origins, dirs):
        """KDTree::intersect over a batch, host buffers: (tid int32, dist float32)."""
        r = rays_to_array(origins, dirs)
        n = len(r)
        tid = np.empty(n, np.int32)
        dist = np.empty(n, np.float32)
        self._ck(self._L.rx_trace_closest(self.h, _capi.ptr(r), n, _capi.ptr(tid), _capi.ptr(dist)))
        return tid, dist

    def trace_closest_rays(self, rays: np.ndarray, tid: np.ndarray, dist: np.ndarray):
        """Host-buffer call on pre-packed rx_ray records (e.g. pinned memory)."""
        self._ck(self._L.rx_trace_closest(self.h, _capi.ptr(rays), len(rays), _capi.ptr(tid), _capi.ptr(dist)))

    def trace_closest_device(self, d_rays, n: int, d_tid, d_dist, stream=None):
        """Device buffers. ``stream``: None = the context's stream, otherwise a
        cudaStream_t handle (0 = the legacy default stream, e.g. torch's default)."""
        self._ck(self._L.rx_trace_closest_device(self.h, _capi.ptr(d_rays), n, _capi.ptr(d_tid), _capi.ptr(d_dist),
                                                 _capi.stream_arg(stream)))

    def trace_reforder_device(self, d_rays, n: int, d_tid, d_dist, stream=None):
        self._ck(self._L.rx_trace_closest_reforder_device(self.h, _capi.ptr(d_rays), n, _capi.ptr(d_tid),
                                                          _capi.ptr(d_dist), _capi.stream_arg(stream)))

    # -- rendering -------------------------------------------------------------------
    def render_pt(self, camera: "scenes.Camera", spp: int, max_depth: int = 8, nee: bool = False, rr_mode: int = 0,
                  seed: int = 1, paths_per_pass: int = 0, want_sq: bool = False, guided: bool = False,
                  time_budget_s: float = 0.0):
        """PathTracer (nee=False) or PathTracerTest (nee=True) renderPixels for ``spp``
        samples: returns (mean (H,W,3) float64, mean of squares or None, stats dict).
        guided: one-sample MIS with the guiding network (guide_init first; PathTracer only).
        time_budget_s > 0: stop after the pass during which that much wall time passed
        (spp is then the cap; stats["paths"] = pixel samples done, each pixel's mean over
        its own samples)."""
        cam = camera_struct(camera)
        o = rx_pt_options(spp, max_depth, rr_mode, int(bool(nee)), seed, paths_per_pass, 1 if guided else 0,
                          float(time_budget_s), 0)
        h, w = camera.height, camera.width
        film = np.zeros((h, w, 3), np.float64)
        sq = np.zeros((h, w, 3), np.float64) if want_sq else None
        st = rx_render_stats()
        self._ck(self._L.rx_render_pt(self.h, ctypes.byref(cam), ctypes.byref(o), _capi.ptr(film), _capi.ptr(sq),
                                      ctypes.byref(st)))
        return film, sq, dict(extension_rays=st.extension_rays, shadow_rays=st.shadow_rays, paths=st.paths, ms=st.ms)

    def render_pt_batch(self, items, paths_per_pass: int = 0, use_graph: bool = True, autotune: bool = False):
        """Renders several scenes in one wavefront. items: list of (Context, Camera,
        dict(spp, max_depth, rr_mode, nee, seed, guided)); guided items use their
        context's network (guide_init on that context). Returns (list of (H,W,3) means,
        stats)."""
        arr = (_capi.rx_batch_item * len(items))()
        films = []
        for k, (ctx, cam, o) in enumerate(items):
            film = np.zeros((cam.height, cam.width, 3), np.float64)
            films.append(film)
            arr[k].scene = ctx.h
            arr[k].camera = camera_struct(cam)
            arr[k].options = rx_pt_options(o.get("spp", 16), o.get("max_depth", 8), o.get("rr_mode", 0),
                                           int(bool(o.get("nee", False))), o.get("seed", 1), 0,
                                           1 if o.get("guided", False) else 0)
            arr[k].film_rgb = film.ctypes.data
        bo = _capi.rx_batch_options(paths_per_pass, int(use_graph), int(autotune), 0, 0, 0)
        st = rx_render_stats()
        self._ck(self._L.rx_render_pt_batch(self.h, arr, len(items), ctypes.byref(bo), ctypes.byref(st)))
        return films, dict(extension_rays=st.extension_rays, shadow_rays=st.shadow_rays, paths=st.paths, ms=st.ms,
                           blocks_per_sm=bo.chosen_blocks_per_sm, stack=bo.chosen_stack,
                           paths_per_pass=bo.chosen_paths_per_pass)

    def render_vcm(self, camera: "scenes.Camera", iterations: int, radius: float, alpha: float = 0.6667,
                   max_depth: int = 8, light_paths: int = 0, seed: int = 1, full_path_mis: bool = False,
                   time_budget_s: float = 0.0):
        """VCMTracer renderPixels for ``iterations``: returns (mean (H,W,3) float64, stats).
        ``full_path_mis`` evaluates merges with the reference's whole-path loops
        (RX_VCM_FULL_PATH_MIS) instead of the per-subpath records. ``time_budget_s`` > 0
        stops after the iteration during which that much wall time passed (the mean is
        over the iterations done: stats["paths"] / pixels)."""
        cam = camera_struct(camera)
        o = rx_vcm_options(iterations, max_depth, light_paths, 1 if full_path_mis else 0, radius, alpha, seed,
                           float(time_budget_s), 0)
        film = np.zeros((camera.height, camera.width, 3), np.float64)
        st = rx_render_stats()
        self._ck(self._L.rx_render_vcm(self.h, ctypes.byref(cam), ctypes.byref(o), _capi.ptr(film), ctypes.byref(st)))
        return film, dict(rays=st.extension_rays, shadow_rays=st.shadow_rays, merges=st.merges, paths=st.paths,
                          ms=st.ms, merge_ms=st.merge_ms, merge_queries=st.merge_queries, photons=st.photons)

    def render_bpt(self, camera: "scenes.Camera", iterations: int, max_depth: int = 8, seed: int = 1,
                   full_path_mis: bool = False, time_budget_s: float = 0.0):
        """BidirectionalPathTracer renderPixels for ``iterations`` samples per pixel:
        returns (mean (H,W,3) float64, stats). ``full_path_mis`` evaluates connections with
        the reference's whole-path loops (RX_VCM_FULL_PATH_MIS). ``time_budget_s`` as
        render_vcm."""
        cam = camera_struct(camera)
        o = rx_bpt_options(iterations, max_depth, 1 if full_path_mis else 0, float(time_budget_s), seed)
        film = np.zeros((camera.height, camera.width, 3), np.float64)
        st = rx_render_stats()
        self._ck(self._L.rx_render_bpt(self.h, ctypes.byref(cam), ctypes.byref(o), _capi.ptr(film), ctypes.byref(st)))
        return film, dict(rays=st.extension_rays, shadow_rays=st.shadow_rays, paths=st.paths, ms=st.ms)

    def render_pm(self, camera: "scenes.Camera", iterations: int, radius: float, max_depth: int = 8,
                  light_paths: int = 0, alpha: float = 0.0, seed: int = 1, time_budget_s: float = 0.0):
        """PhotonMap renderPixels for ``iterations``: returns (mean (H,W,3) float64, stats);
        ``alpha`` 0 is the reference's 2/3, ``light_paths`` 0 is width * height;
        ``time_budget_s`` as render_vcm."""
        cam = camera_struct(camera)
        o = rx_pm_options(iterations, max_depth, light_paths, 0, radius, alpha, seed, float(time_budget_s), 0)
        film = np.zeros((camera.height, camera.width, 3), np.float64)
        st = rx_render_stats()
        self._ck(self._L.rx_render_pm(self.h, ctypes.byref(cam), ctypes.byref(o), _capi.ptr(film), ctypes.byref(st)))
        return film, dict(rays=st.extension_rays, photons=st.merges, paths=st.paths, ms=st.ms)

    def set_trace_config(self, variant: int = 4, blocks_per_sm: int = 12):
        self._ck(self._L.rx_trace_set_config(self.h, variant, blocks_per_sm))

    def set_snapshots(self, every_s: float, fn=None):
        """Convergence snapshots of the following renders (rx_set_snapshots): fn(elapsed_s,
        samples, mean (H,W,3) float64 copy) after the pass or iteration during which the
        elapsed wall time reached each next multiple of every_s; every_s = 0 or fn None
        turns them off."""
        if fn is None or every_s <= 0:
            self._snap_cb = None
            self._ck(self._L.rx_set_snapshots(self.h, 0.0, _capi.SNAPSHOT_FN(), None))
            return

        def cb(_user, elapsed, samples, film, w, h):
            fn(elapsed, samples, np.ctypeslib.as_array(film, shape=(h * w * 3,)).reshape(h, w, 3).copy())

        self._snap_cb = _capi.SNAPSHOT_FN(cb)  # kept alive while the library may call it
        self._ck(self._L.rx_set_snapshots(self.h, float(every_s), self._snap_cb, None))

    def set_trace_staging(self, chunk_rays: int = 0):
        """Rays per staged chunk of the host-buffer call (0 = default 2^22)."""
        self._ck(self._L.rx_trace_set_staging(self.h, int(chunk_rays)))

    def set_trace_binning(self, cell_bits: int = 4, dir_bits: int = 4, dir_map: int = 1):
        """Binning key of the closest-hit batch: 2^cell_bits origin cells per axis, then a
        direction bin: 2^dir_bits levels per component (dir_map 0) or a 2^dir_bits square
        grid over the octahedral map (dir_map 1)."""
        self._ck(self._L.rx_trace_set_binning(self.h, int(cell_bits), int(dir_bits), int(dir_map)))

    def set_trace_options(self, check_mode: int = 1, bin_min: int = 1 << 18, walk_stack: int = 0):
        """Visibility check of each winner (1 = thread per ray, 0 = warp per ray), the
        batch size from which rays are binned before the walk (0 = never) and the walk
        stack depth (0 = automatic, 32 or 64)."""
        self._ck(self._L.rx_trace_set_options(self.h, int(check_mode), int(bin_min), int(walk_stack)))

    def set_trace_timing(self, max_calls: int):
        """Record per-kernel CUDA events for the next ``max_calls`` device trace calls."""
        self._ck(self._L.rx_trace_set_timing(self.h, int(max_calls)))

    def read_trace_timing(self) -> np.ndarray:
        """(calls, 3) device milliseconds: walk, visibility check, re-walk."""
        n = ctypes.c_int32(0)
        self._ck(self._L.rx_trace_read_timing(self.h, None, ctypes.byref(n)))
        out = np.zeros((n.value, 3), np.float32)
        if n.value:
            self._ck(self._L.rx_trace_read_timing(self.h, _capi.ptr(out), ctypes.byref(n)))
        return out

    def diag_umma_gemm(self, a: np.ndarray, b: np.ndarray, a_mn: bool = False, b_mn: bool = False) -> np.ndarray:
        """Tensor-core layout self-test: A (M x K) and B (N x K) as bf16 bit patterns
        (uint16); returns all 128 tensor-memory lanes x N columns of A @ B.T (float32)."""
        a = np.ascontiguousarray(a, np.uint16)
        b = np.ascontiguousarray(b, np.uint16)
        (m, k), n = a.shape, b.shape[0]
        assert b.shape[1] == k
        out = np.zeros((128, n), np.float32)
        self._ck(self._L.rx_diag_umma_gemm(self.h, m, n, k, int(a_mn), int(b_mn), _capi.ptr(a), _capi.ptr(b),
                                           _capi.ptr(out)))
        return out

    def diag_umma_rate(self, n: int, count: int = 256) -> tuple:
        """Tensor-core issue rate: SM clock cycles per back-to-back BF16 MMA of
        M = 128, K = 16 and N = n (64, 128 or 256) from one thread, (to the last issue, to
        completion)."""
        issue, done = ctypes.c_double(), ctypes.c_double()
        self._ck(self._L.rx_diag_umma_rate(self.h, int(n), int(count), ctypes.byref(issue), ctypes.byref(done)))
        return issue.value, done.value

    # ---- learned guiding ---------------------------------------------------------
    def guide_init(self, learning_rate: float = 5e-3, bsdf_fraction: float = 0.5, batch: int = 1 << 18,
                   train_passes: int = 4, steps_per_pass: int = 4, warmup_passes: int = 0, seed: int = 1, box=None):
        """Creates the guiding network (seeded weights). box = (min xyz, max xyz) of the
        position encoding, default the scene bounds. The first warmup_passes passes of a
        guided render sample by the BSDF alone; the first train_passes passes train."""
        o = _capi.rx_guide_options(learning_rate, bsdf_fraction, batch, train_passes, steps_per_pass, warmup_passes,
                                   seed)
        b = None if box is None else np.ascontiguousarray(np.concatenate([box[0], box[1]]), np.float32)
        self._ck(self._L.rx_guide_init(self.h, ctypes.byref(o), _capi.ptr(b)))

    def guide_params(self) -> np.ndarray:
        out = np.zeros(21504, np.float32)
        self._ck(self._L.rx_guide_get_params(self.h, _capi.ptr(out)))
        return out

    def guide_set_params(self, params: np.ndarray):
        p = np.ascontiguousarray(params, np.float32)
        assert p.shape == (21504,)
        self._ck(self._L.rx_guide_set_params(self.h, _capi.ptr(p)))

    def guide_eval(self, recs: np.ndarray):
        """Forward pass on (n, 16) records: (raw outputs (n, 40), mixture pdf of wi (n,))."""
        r = np.ascontiguousarray(recs, np.float32)
        n = len(r)
        raw = np.zeros((n, 40), np.float32)
        pdf = np.zeros(n, np.float32)
        self._ck(self._L.rx_guide_eval(self.h, _capi.ptr(r), n, _capi.ptr(raw), _capi.ptr(pdf)))
        return raw, pdf

    def guide_eval_device(self, d_recs, n: int, d_raw=None, d_pdf=None, stream=None):
        """Forward pass on n device records (pointers or tensors), enqueued on ``stream``."""
        self._ck(self._L.rx_guide_eval_device(self.h, _capi.ptr(d_recs), n, _capi.ptr(d_raw), _capi.ptr(d_pdf),
                                              _capi.stream_arg(stream)))

    def guide_gradient(self, recs: np.ndarray):
        """(loss, gradient (21504,)) of the batch loss on (n, 16) records, no update."""
        r = np.ascontiguousarray(recs, np.float32)
        g = np.zeros(21504, np.float32)
        loss = ctypes.c_float(0)
        self._ck(self._L.rx_guide_gradient(self.h, _capi.ptr(r), len(r), _capi.ptr(g), ctypes.byref(loss)))
        return float(loss.value), g

    def guide_train_step(self, d_recs, n: int, stream=None, want_loss: bool = True):
        """One Adam step on n device records (a pointer or tensor)."""
        loss = ctypes.c_float(0)
        self._ck(self._L.rx_guide_train_step(self.h, _capi.ptr(d_recs), n,
                                             ctypes.byref(loss) if want_loss else None, _capi.stream_arg(stream)))
        return float(loss.value) if want_loss else None

    def counters(self, reset: bool = False) -> dict:
        out = np.zeros(4, np.uint64)
        self._ck(self._L.rx_trace_counters(self.h, _capi.ptr(out), int(reset)))
        return dict(exact_box_tests=int(out[1]), eager_retraces=int(out[2]), errors=int(out[3]))


def camera_struct(c: "scenes.Camera") -> rx_camera:
    r = rx_camera()
    r.width, r.height, r.sight_dist = c.width, c.height, c.sight_dist
    r.position[:] = c.position
    r.focus[:] = c.focus
    r.up[:] = c.up
    return r


def objects_from_scene(scene: "scenes.Scene"):
    objs = []
    off = 0
    for o in scene.objects:
        m = o.material
        ro = rx_object()
        ro.tri_begin, ro.tri_count, ro.material = off, len(o.tris), m.kind
        ro.has_vertex_normals = 0 if o.normals is None else 1
        ro.color[:] = m.color
        ro.coeff = m.coeff
        ro.diffuse_color[:] = m.diffuse_color
        ro.ior = m.ior
        ro.sigma_s[:] = m.sigma_s
        ro.sigma_a[:] = m.sigma_a
        ro.g = m.g
        ro.decay[:] = m.decay
        ro.step_size = m.step_size
        objs.append(ro)
        off += len(o.tris)
    return objs


class KDTree:
    """Host mirror of the reference's KDTree (include/KDTree.h:10-59) backed by the GPU.

    ``vertexPositionList`` (n,3) and ``triangleList`` (m,3) are filled by the caller,
    ``build()`` uploads and builds, ``intersect(origins, dirs)`` returns per ray
    ``(dist, triangleID)`` with dist = -1 on a miss (KDTree.h:50)."""

    def __init__(self, device: int = 0, split_policy: int = SPLIT_GCC):
        self.vertexPositionList = np.zeros((0, 3), np.float32)
        self.triangleList = np.zeros((0, 3), np.uint32)
        self.split_policy = split_policy
        self._ctx = Context(device)

    def build(self):
        self._ctx.set_geometry(self.vertexPositionList, self.triangleList)
        self._ctx.build_accel(self.split_policy)

    def intersect(self, origins, dirs):
        tid, dist = self._ctx.trace_closest(origins, dirs)
        return dist, tid

    def serializeForGPU(self):
        return reftree_serialize(self.vertexPositionList, self.triangleList, self.split_policy)
