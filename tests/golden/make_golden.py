"""Generates the closest-hit golden fixtures from the reference's own KDTree.

Runs only where the reference sources are mounted: builds oracle/_ref/hit_driver from
them (oracle/ref/Makefile), then for each case writes ``hit_<case>.npz`` with the rays,
the reference's (tid, dist) answers and its serialized tree (KDTree::serializeForGPU).
Scenes come from renderx_gb300.scenes with fixed seeds; small scenes also store their
geometry so the fixture stands alone.

    python tests/golden/make_golden.py [REF_DIR]
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from renderx_gb300 import scenes, sceneio  # noqa: E402

CASES = {
    # name: (n_spheres, subdiv, scene seed, random rays, store geometry)
    "cornell": (0, 0, 0, 4096, True),
    "spheres4": (4, 3, 3, 4096, True),
    "spheres20": (20, 4, 5, 2048, False),
}


def geometry_hash(verts: np.ndarray, tris: np.ndarray) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(verts, np.float32).tobytes())
    h.update(np.ascontiguousarray(tris, np.uint32).tobytes())
    return h.hexdigest()


def make_scene(ns: int, sub: int, seed: int):
    sc = scenes.sphere_field(ns, sub, seed=seed, width=64, height=64) if ns else scenes.cornell_box(64, 64)
    return sc.flatten()


def stress_rays(verts: np.ndarray, tris: np.ndarray, n: int, seed: int):
    """Rays that stress ties, zero direction components and surface origins."""
    rng = np.random.default_rng(seed)
    R = scenes.ROOM
    o_list, d_list = [], []
    # 1. aimed exactly at shared vertices and edge midpoints (equal-distance candidates)
    pick = rng.integers(0, len(tris), n // 4)
    for k, t in enumerate(pick):
        a, b = verts[tris[t, k % 3]], verts[tris[t, (k + 1) % 3]]
        target = a if k % 2 == 0 else (a + b) * np.float32(0.5)
        o = rng.uniform(0.2, R - 0.2, 3).astype(np.float32)
        d = (target - o).astype(np.float64)
        d /= np.linalg.norm(d)
        o_list.append(o)
        d_list.append(d.astype(np.float32))
    # 2. axis-aligned and planar directions (reference skips faces where d[axis] == 0)
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                     [0.6, 0, 0.8], [0, -0.8, 0.6], [0.8, 0.6, 0]], np.float32)
    for k in range(n // 4):
        o_list.append(rng.uniform(0.0, R, 3).astype(np.float32))
        d_list.append(axes[k % len(axes)])
    # 3. origins on triangles (t = 0 candidates) and just off them
    pick = rng.integers(0, len(tris), n // 4)
    for t in pick:
        w = rng.dirichlet([1, 1, 1])
        p = (w[0] * verts[tris[t, 0]] + w[1] * verts[tris[t, 1]] + w[2] * verts[tris[t, 2]]).astype(np.float32)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        o_list.append(p)
        d_list.append(d.astype(np.float32))
    # 4. grazing rays in the floor plane and from outside the room
    for k in range(n - 3 * (n // 4)):
        if k % 2 == 0:
            o = np.array([rng.uniform(0, R), 0.0, rng.uniform(0, R)], np.float32)
            phi = rng.uniform(0, 2 * np.pi)
            d = np.array([np.cos(phi), 0.0, np.sin(phi)], np.float32)
        else:
            o = rng.uniform(-3.0, R + 3.0, 3).astype(np.float32)
            d = (rng.uniform(0.5, R - 0.5, 3) - o).astype(np.float64)
            d = (d / np.linalg.norm(d)).astype(np.float32)
        o_list.append(o)
        d_list.append(d)
    return np.array(o_list, np.float32), np.array(d_list, np.float32)


def run_reference(ref_bin: str, verts, tris, o, d):
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "c")
        np.ascontiguousarray(verts, np.float32).tofile(p + ".v")
        np.ascontiguousarray(tris, np.uint32).tofile(p + ".t")
        np.concatenate([o, d], 1).astype(np.float32).tofile(p + ".r")
        subprocess.run([ref_bin, p + ".v", p + ".t", p + ".r", p], check=True, capture_output=True,
                       env={**os.environ, "OMP_NUM_THREADS": "8"})
        return (np.fromfile(p + ".tid.i32", np.int32), np.fromfile(p + ".dist.f32", np.float32),
                np.fromfile(p + ".nodes.f32", np.float32).reshape(-1, 12), np.fromfile(p + ".leaf.f32", np.float32))


# Path-tracing goldens: (scene function, renderer mode, max depth, spp). The reference
# renders through its own ConfigManager from the XML/OBJ files sceneio writes.
RENDER_CASES = {
    "cornell_pt": ("cornell_box", "pt", 8, 4096),
    "cornell_nee": ("cornell_box", "ptnee", 8, 4096),
    "spheres_pt": ("material_spheres", "pt", 8, 4096),
    "spheres_nee": ("material_spheres", "ptnee", 8, 4096),
    "medium_pt": ("medium_scene", "pt", 8, 4096),
    "medium_nee": ("medium_scene", "ptnee", 8, 4096),
}


def render_scene(name: str, w: int = 64, h: int = 64) -> scenes.Scene:
    return getattr(scenes, name)(w, h)


def _selected(case: str) -> bool:
    only = [a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")]
    return not only or case in only[0].split(",")


def make_render_goldens(ref_pt: str):
    for case, (scene_fn, mode, depth, spp) in RENDER_CASES.items():
        if not _selected(case):
            continue
        sc = render_scene(scene_fn)
        f = sc.flatten()
        with tempfile.TemporaryDirectory() as td:
            cfg = sceneio.write_config(sc, td, "PTtest" if mode == "ptnee" else "PT", depth)
            pre = os.path.join(td, "out")
            out = subprocess.run([ref_pt, cfg, mode, str(spp), pre, "8"], check=True, capture_output=True,
                                 text=True, cwd=td).stdout.strip().splitlines()[-1].split()
            s1 = np.fromfile(pre + ".sum.f64").reshape(sc.camera.height, sc.camera.width, 3)
            s2 = np.fromfile(pre + ".sq.f64").reshape(sc.camera.height, sc.camera.width, 3)
        mean = s1 / spp
        var = np.maximum(s2 / spp - mean * mean, 0.0) * spp / (spp - 1)
        path = os.path.join(HERE, f"render_{case}.npz")
        np.savez_compressed(path, mean=mean.astype(np.float32), stderr=np.sqrt(var / spp).astype(np.float32),
                            spp=np.int64(spp), max_depth=np.int64(depth), mode=np.array(mode),
                            scene=np.array(scene_fn), segments=np.int64(out[3]), seconds=np.float64(out[4]),
                            geometry_sha256=np.array(geometry_hash(f["verts"], f["tris"])))
        print(f"{path}: {spp} spp, mean {mean.mean(axis=(0, 1))}, {out[4]} s")


# VCM goldens: (scene function, max depth, iterations per estimate, independent
# estimates, initial radius, alpha). One reference process per estimate.
VCM_CASES = {
    "cornell_vcm": ("cornell_box", 8, 8, 64, 0.0963, 0.75),
    "spheres_vcm": ("material_spheres", 8, 8, 48, 0.0963, 0.75),
    "medium_vcm": ("medium_scene", 8, 8, 48, 0.0963, 0.75),
    # an eighth of the radius: merging's blur bias is negligible, so the GPU's renders with
    # another light-path count than width * height have the same expectation
    "cornell_vcm_r8": ("cornell_box", 8, 8, 64, 0.0963 / 8, 0.75),
    "spheres_vcm_r8": ("material_spheres", 8, 8, 48, 0.0963 / 8, 0.75),
    "medium_vcm_r8": ("medium_scene", 8, 8, 48, 0.0963 / 8, 0.75),
}


def make_vcm_goldens(ref_vcm: str):
    for case, (scene_fn, depth, iters, runs, r0, alpha) in VCM_CASES.items():
        if not _selected(case):
            continue
        sc = render_scene(scene_fn)
        f = sc.flatten()
        imgs = []
        secs = 0.0
        with tempfile.TemporaryDirectory() as td:
            cfg = sceneio.write_config(sc, td, "VCM", depth, radius=r0)
            for run in range(runs):
                pre = os.path.join(td, f"out{run}")
                out = subprocess.run([ref_vcm, cfg, str(iters), str(run), str(r0), str(alpha), pre, "8"], check=True,
                                     capture_output=True, text=True, cwd=td).stdout.strip().splitlines()[-1].split()
                secs += float(out[-1])
                imgs.append(np.fromfile(pre + ".img.f64").reshape(sc.camera.height, sc.camera.width, 3))
        imgs = np.array(imgs)
        mean = imgs.mean(axis=0)
        stderr = imgs.std(axis=0, ddof=1) / np.sqrt(runs)
        # standard errors of 4x4-block means from the runs themselves (merging correlates
        # neighbouring pixels, so they are not the per-pixel errors combined)
        h, w, _ = mean.shape
        blocks = imgs.reshape(runs, h // 4, 4, w // 4, 4, 3).mean(axis=(2, 4))
        block_stderr = blocks.std(axis=0, ddof=1) / np.sqrt(runs)
        path = os.path.join(HERE, f"render_{case}.npz")
        np.savez_compressed(path, mean=mean.astype(np.float32), stderr=stderr.astype(np.float32),
                            block_stderr=block_stderr.astype(np.float32),
                            runs=np.int64(runs), iterations=np.int64(iters), max_depth=np.int64(depth),
                            radius=np.float64(r0), alpha=np.float64(alpha), scene=np.array(scene_fn),
                            seconds=np.float64(secs), geometry_sha256=np.array(geometry_hash(f["verts"], f["tris"])))
        print(f"{path}: {runs} x {iters} iterations, mean {mean.mean(axis=(0, 1))}, {secs:.1f} s", flush=True)


# BidirectionalPathTracer goldens: (scene function, max depth, samples per estimate,
# independent estimates). One reference process per estimate.
BPT_CASES = {
    "cornell_bpt": ("cornell_box", 8, 8, 64),
    "spheres_bpt": ("material_spheres", 8, 8, 48),
    "medium_bpt": ("medium_scene", 8, 8, 48),
}


def make_bpt_goldens(ref_bpt: str):
    for case, (scene_fn, depth, spp, runs) in BPT_CASES.items():
        if not _selected(case):
            continue
        sc = render_scene(scene_fn)
        f = sc.flatten()
        imgs = []
        secs = 0.0
        with tempfile.TemporaryDirectory() as td:
            cfg = sceneio.write_config(sc, td, "BPT", depth)
            for run in range(runs):
                pre = os.path.join(td, f"out{run}")
                out = subprocess.run([ref_bpt, cfg, str(spp), str(run), pre, "8"], check=True, capture_output=True,
                                     text=True, cwd=td).stdout.strip().splitlines()[-1].split()
                secs += float(out[-1])
                imgs.append(np.fromfile(pre + ".img.f64").reshape(sc.camera.height, sc.camera.width, 3))
        imgs = np.array(imgs)
        mean = imgs.mean(axis=0)
        stderr = imgs.std(axis=0, ddof=1) / np.sqrt(runs)
        path = os.path.join(HERE, f"render_{case}.npz")
        np.savez_compressed(path, mean=mean.astype(np.float32), stderr=stderr.astype(np.float32),
                            runs=np.int64(runs), iterations=np.int64(spp), max_depth=np.int64(depth),
                            scene=np.array(scene_fn), seconds=np.float64(secs),
                            geometry_sha256=np.array(geometry_hash(f["verts"], f["tris"])))
        print(f"{path}: {runs} x {spp} spp, mean {mean.mean(axis=(0, 1))}, {secs:.1f} s", flush=True)


# PhotonMap goldens: (scene function, max depth, iterations per estimate, independent
# estimates, base radius, medium ray-marching step). One reference process per estimate.
PM_CASES = {
    "cornell_pm": ("cornell_box", 8, 8, 64, 0.0963, 0.01),
    "spheres_pm": ("material_spheres", 8, 8, 48, 0.0963, 0.01),
    "medium_pm": ("medium_scene", 8, 8, 48, 0.0963, 0.01),
}


def pm_scene(scene_fn: str, step: float):
    sc = render_scene(scene_fn)
    for o in sc.objects:
        if o.material.kind == scenes.VPM:
            o.material.step_size = step
    return sc


def make_pm_goldens(ref_pm: str):
    for case, (scene_fn, depth, iters, runs, r0, step) in PM_CASES.items():
        if not _selected(case):
            continue
        sc = pm_scene(scene_fn, step)
        f = sc.flatten()
        imgs = []
        secs = 0.0
        with tempfile.TemporaryDirectory() as td:
            cfg = sceneio.write_config(sc, td, "PM", depth, radius=r0)
            for run in range(runs):
                pre = os.path.join(td, f"out{run}")
                out = subprocess.run([ref_pm, cfg, str(iters), str(run), str(r0), pre, "8"], check=True,
                                     capture_output=True, text=True, cwd=td).stdout.strip().splitlines()[-1].split()
                secs += float(out[-1])
                imgs.append(np.fromfile(pre + ".img.f64").reshape(sc.camera.height, sc.camera.width, 3))
        imgs = np.array(imgs)
        mean = imgs.mean(axis=0)
        stderr = imgs.std(axis=0, ddof=1) / np.sqrt(runs)
        path = os.path.join(HERE, f"render_{case}.npz")
        np.savez_compressed(path, mean=mean.astype(np.float32), stderr=stderr.astype(np.float32),
                            runs=np.int64(runs), iterations=np.int64(iters), max_depth=np.int64(depth),
                            radius=np.float64(r0), step_size=np.float64(step), scene=np.array(scene_fn),
                            seconds=np.float64(secs), geometry_sha256=np.array(geometry_hash(f["verts"], f["tris"])))
        print(f"{path}: {runs} x {iters} iterations, mean {mean.mean(axis=(0, 1))}, {secs:.1f} s", flush=True)


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref = args[0] if args else (os.environ.get("RENDERX_REFERENCE") or
                                os.path.join(os.path.dirname(ROOT), "reference"))
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={ref}"], check=True)
    if "--bpt-only" in sys.argv:
        make_bpt_goldens(os.path.join(ROOT, "oracle", "_ref", "bpt_driver"))
        return
    if "--pm-only" in sys.argv:
        make_pm_goldens(os.path.join(ROOT, "oracle", "_ref", "pm_driver"))
        return
    if "--vcm-only" not in sys.argv:
        make_render_goldens(os.path.join(ROOT, "oracle", "_ref", "pt_driver"))
    make_vcm_goldens(os.path.join(ROOT, "oracle", "_ref", "vcm_driver"))
    make_bpt_goldens(os.path.join(ROOT, "oracle", "_ref", "bpt_driver"))
    make_pm_goldens(os.path.join(ROOT, "oracle", "_ref", "pm_driver"))
    if "--render-only" in sys.argv or "--vcm-only" in sys.argv:
        return
    ref_bin = os.path.join(ROOT, "oracle", "_ref", "hit_driver")
    for name, (ns, sub, seed, nrand, store) in CASES.items():
        f = make_scene(ns, sub, seed)
        v, t = f["verts"], f["tris"]
        o1, d1 = scenes.hit_rays(nrand, seed=100 + seed)
        o2, d2 = stress_rays(v, t, nrand, seed=200 + seed)
        o = np.concatenate([o1, o2])
        d = np.concatenate([d1, d2])
        tid, dist, nodes, leaf = run_reference(ref_bin, v, t, o, d)
        out = dict(origins=o, dirs=d, tid=tid, dist=dist, nodes=nodes, leaf=leaf,
                   params=np.array([ns, sub, seed], np.int64), geometry_sha256=np.array(geometry_hash(v, t)))
        if store:
            out.update(verts=v, tris=t)
        path = os.path.join(HERE, f"hit_{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {len(o)} rays, {len(t)} tris, {len(nodes)} nodes, hit rate {(tid >= 0).mean():.3f}, "
              f"{os.path.getsize(path) // 1024} KiB")


if __name__ == "__main__":
    main()
