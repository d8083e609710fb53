"""ORACLE — test infrastructure only.

CPU restatement of the reference's light-transport path, compiled from
``oracle/*.cpp`` into ``oracle/liboracle.so``: the triangle KDTree (reference
src/KDTree.cpp; ``RefTree``) and the PathTracer estimator with the surface materials
(src/PathTracer.cpp, src/MCRenderer.cpp, the material code; ``RefPathTracer``). The
guiding network's FP64 restatement is ``oracle.guide_mlp``. Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg may import this package; it checks results and times
the CPU baseline, and is never the thing measured or shipped.

Parity pins: ``tests/test_oracle_golden.py`` checks this restatement against golden
fixtures produced by the reference's own code compiled from its sources
(``oracle/ref/``, script ``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

SPLIT_GCC = 0   # reference as built by GCC/libstdc++: always splits on x
SPLIT_BEST = 1  # reference's intended best-axis choice (libc++/MSVC builds)


def build(force: bool = False) -> str:
    path = os.path.join(_HERE, "liboracle.so")
    srcs = [os.path.join(_HERE, f) for f in os.listdir(_HERE) if f.endswith(".cpp")]
    if force or not os.path.exists(path) or any(os.path.getmtime(s) > os.path.getmtime(path) for s in srcs):
        subprocess.run(["make", "-s", "-C", _HERE, "-B"], check=True)
    return path


def lib():
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(build())
        P = ctypes.c_void_p
        L.rxo_tree_build.restype = P
        L.rxo_tree_build.argtypes = [P, ctypes.c_uint32, P, ctypes.c_uint32, ctypes.c_int]
        L.rxo_tree_free.argtypes = [P]
        for f in ("rxo_tree_num_nodes", "rxo_tree_num_leaf_tris"):
            getattr(L, f).restype = ctypes.c_uint32
            getattr(L, f).argtypes = [P]
        L.rxo_tree_max_depth.restype = ctypes.c_int
        L.rxo_tree_max_depth.argtypes = [P]
        L.rxo_tree_serialize.argtypes = [P, P, P]
        L.rxo_trace.argtypes = [P, P, ctypes.c_uint32, P, P, ctypes.c_int]
        L.rxo_trace_unboxed.argtypes = [P, P, ctypes.c_uint32, P, P, ctypes.c_int]
        L.rxo_box_test.restype = ctypes.c_float
        L.rxo_box_test.argtypes = [P, P, P, P]
        L.rxo_num_threads.restype = ctypes.c_int
        L.rxo_pt_render.restype = ctypes.c_uint64
        L.rxo_pt_render.argtypes = [P, P, P, P, ctypes.c_uint32, P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint64, ctypes.c_int, P, P]
        _LIB = L
    return _LIB


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class RefTree:
    """The reference's triangle tree, restated (KDTree::build / splitBest)."""

    def __init__(self, verts: np.ndarray, tris: np.ndarray, policy: int = SPLIT_GCC):
        self._v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        self._t = np.ascontiguousarray(tris, np.uint32).reshape(-1, 3)
        self.h = lib().rxo_tree_build(_p(self._v), len(self._v), _p(self._t), len(self._t), policy)
        if not self.h:
            raise ValueError("empty scene")

    def __del__(self):
        if getattr(self, "h", None):
            lib().rxo_tree_free(self.h)
            self.h = None

    @property
    def num_nodes(self) -> int:
        return lib().rxo_tree_num_nodes(self.h)

    @property
    def max_depth(self) -> int:
        return lib().rxo_tree_max_depth(self.h)

    def serialize(self):
        """(nodes (n,12) f32, leaf_tid (m,) f32) in serializeForGPU's layout."""
        n = self.num_nodes
        m = lib().rxo_tree_num_leaf_tris(self.h)
        nodes = np.zeros((n, 12), np.float32)
        leaf = np.zeros(m, np.float32)
        lib().rxo_tree_serialize(self.h, _p(nodes), _p(leaf))
        return nodes, leaf

    def trace(self, origins: np.ndarray, dirs: np.ndarray, threads: int = 0):
        """Closest hit per ray: (tid int32 with -1 on miss, dist float32)."""
        return self._run(lib().rxo_trace, origins, dirs, threads)

    def trace_unboxed(self, origins: np.ndarray, dirs: np.ndarray, threads: int = 0):
        """Closest hit over every triangle, the tree's box tests ignored (same tie
        order). Rays where this differs from trace() are those whose closest triangle
        the reference's box tests hide."""
        return self._run(lib().rxo_trace_unboxed, origins, dirs, threads)

    def _run(self, fn, origins, dirs, threads):
        r = np.ascontiguousarray(np.concatenate([np.asarray(origins, np.float32).reshape(-1, 3),
                                                 np.asarray(dirs, np.float32).reshape(-1, 3)], 1))
        n = len(r)
        tid = np.empty(n, np.int32)
        dist = np.empty(n, np.float32)
        fn(self.h, _p(r), n, _p(tid), _p(dist), threads)
        return tid, dist


class _PtObject(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("color", ctypes.c_float * 3), ("coeff", ctypes.c_float),
                ("diffuse_color", ctypes.c_float * 3), ("ior", ctypes.c_float), ("decay", ctypes.c_float * 3),
                ("has_normals", ctypes.c_uint32)]


class _PtCamera(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("sight_dist", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("position", ctypes.c_float * 3), ("focus", ctypes.c_float * 3),
                ("up", ctypes.c_float * 3)]


class RefPathTracer:
    """The reference's PathTracer restated on the CPU (rxo_pt.cpp) over the reference's
    own tree and traversal: surface materials, objects that neither overlap nor nest."""

    def __init__(self, scene, policy: int = SPLIT_GCC, tree: "RefTree | None" = None):
        f = scene.flatten()
        self.tree = tree if tree is not None else RefTree(f["verts"], f["tris"], policy)
        self._tri_obj = np.ascontiguousarray(f["tri_obj"], np.uint32)
        self._normals = np.ascontiguousarray(f["normals"], np.float32)
        objs = (_PtObject * len(scene.objects))()
        for k, o in enumerate(scene.objects):
            m = o.material
            objs[k].kind = m.kind
            objs[k].color[:] = m.color
            objs[k].coeff = m.coeff
            objs[k].diffuse_color[:] = m.diffuse_color
            objs[k].ior = -1.0 if m.kind == 5 else m.ior
            objs[k].decay[:] = m.decay
            objs[k].has_normals = int(f["has_normals"][k])
        self._objs = objs

    def render(self, camera, spp: int, max_depth: int = 8, rr_mode: int = 0, seed: int = 1, crop=None,
               threads: int = 0, want_sq: bool = False):
        """Per-pixel mean over spp samples of the crop (x0, y0, w, h) (default the whole
        image) as (h, w, 3) float64, the mean of squares (want_sq) or None, and the
        number of closest-hit queries traced."""
        x0, y0, w, h = crop if crop is not None else (0, 0, camera.width, camera.height)
        cam = _PtCamera(camera.width, camera.height, camera.sight_dist, 0)
        cam.position[:] = camera.position
        cam.focus[:] = camera.focus
        cam.up[:] = camera.up
        s = np.zeros((h, w, 3), np.float64)
        q = np.zeros((h, w, 3), np.float64) if want_sq else None
        rays = lib().rxo_pt_render(self.tree.h, _p(self._tri_obj), _p(self._normals), ctypes.byref(self._objs),
                                   len(self._objs), ctypes.byref(cam), x0, y0, w, h, spp, max_depth, rr_mode, seed,
                                   threads, _p(s), None if q is None else _p(q))
        return s / spp, (q / spp if q is not None else None), int(rays)


def box_test(mn, mx, o, d) -> float:
    a = [np.ascontiguousarray(x, np.float32) for x in (mn, mx, o, d)]
    return lib().rxo_box_test(*[_p(x) for x in a])


def num_threads() -> int:
    return lib().rxo_num_threads()
