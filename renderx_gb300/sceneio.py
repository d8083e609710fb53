"""Scene files in the reference's own format.

``write_config`` writes a scenes.Scene as the reference's XML + OBJ files: a config
file (``<Config><Scene><path/><name/><camera/></Scene><Renderer>...</Renderer>``,
reference ConfigManager.cpp:166-405), a scene file (``<Scene Name=...>`` with one
``<Object><filePath/><Material>...</Material></Object>`` per object and a
``<Camera Name=...>``, ConfigManager.cpp:25-164, 263-269) and one OBJ per object
(``v``/``vn``/``f a//a b//b c//c``, reference SimpleShape.cpp:44-313). Coordinates are
written with 9 significant digits so float32 values survive the round trip exactly;
objects carry no transform (identity), so world-space vertices equal the OBJ's.

``read_config`` parses the same files back into a scenes.Scene (the host-side mirror of
ConfigManager::load used by tests; the library's C++ loader is the product path).
"""
from __future__ import annotations

import os
import re
import xml.etree.ElementTree as ET

import numpy as np

from . import scenes
from .scenes import DIFFUSE, EMISSIVE, GLOSSY, PHONG, REFLECTIVE, REFRACTIVE, VPM

_TYPE = {DIFFUSE: "Diffuse", GLOSSY: "Glossy", REFRACTIVE: "Refractive", EMISSIVE: "Emissive", PHONG: "Phong",
         REFLECTIVE: "Reflective", VPM: "VPM"}
_KIND = {v: k for k, v in _TYPE.items()}


def _vec(v) -> str:
    return "(" + ", ".join(f"{float(x):.9g}" for x in v) + ")"


def write_obj(path: str, verts: np.ndarray, tris: np.ndarray, normals: np.ndarray | None = None):
    v = np.asarray(verts, np.float32)
    t = np.asarray(tris, np.int64) + 1
    lines = [f"v {a:.9g} {b:.9g} {c:.9g}" for a, b, c in v.tolist()]
    if normals is not None:
        lines += [f"vn {a:.9g} {b:.9g} {c:.9g}" for a, b, c in np.asarray(normals, np.float32).tolist()]
        lines += [f"f {a}//{a} {b}//{b} {c}//{c}" for a, b, c in t.tolist()]
    else:
        lines += [f"f {a} {b} {c}" for a, b, c in t.tolist()]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _material_xml(m: scenes.Material) -> str:
    x = [f"<type>{_TYPE[m.kind]}</type>"]
    if m.kind in (DIFFUSE, GLOSSY, EMISSIVE, REFLECTIVE):
        x.append(f"<color>{_vec(m.color)}</color>")
    if m.kind == GLOSSY:
        x.append(f"<coeff>{m.coeff:.9g}</coeff>")
    if m.kind == REFRACTIVE:
        x.append(f"<coeff>{m.ior:.9g}</coeff>")
        x.append(f"<surfColor>{_vec(m.color)}</surfColor>")
        x.append(f"<decayColor>{_vec(m.decay)}</decayColor>")
    if m.kind == PHONG:
        x.append(f"<GlossyComponent><color>{_vec(m.color)}</color><coeff>{m.coeff:.9g}</coeff></GlossyComponent>")
        x.append(f"<DiffuseComponent><color>{_vec(m.diffuse_color)}</color></DiffuseComponent>")
    if m.kind == VPM:
        x.append(f"<sigma_s>{_vec(m.sigma_s)}</sigma_s><sigma_a>{_vec(m.sigma_a)}</sigma_a>")
        x.append(f"<inrate>{m.ior:.9g}</inrate><g>{m.g:.9g}</g><stepsize>{m.step_size:.9g}</stepsize>")
    return "<Material>" + "".join(x) + "</Material>"


def write_config(scene: scenes.Scene, folder: str, renderer: str = "PT", max_depth: int = 8, radius: float | None = None,
                 name: str = "scene", minutes: int = 1) -> str:
    """Writes config.xml, scene.xml and one OBJ per object into ``folder``; returns the
    config path."""
    os.makedirs(folder, exist_ok=True)
    objs = []
    for i, o in enumerate(scene.objects):
        fn = f"obj{i:04d}.obj"
        write_obj(os.path.join(folder, fn), o.verts, o.tris, o.normals)
        objs.append(f"  <Object Name=\"{o.name}\"><filePath>{fn}</filePath>{_material_xml(o.material)}</Object>")
    c = scene.camera
    cam = (f"  <Camera Name=\"cam\"><width>{c.width}</width><height>{c.height}</height>"
           f"<sightDist>{c.sight_dist}</sightDist><focus>{_vec(c.focus)}</focus>"
           f"<position>{_vec(c.position)}</position><up>{_vec(c.up)}</up></Camera>")
    with open(os.path.join(folder, "scene.xml"), "w") as f:
        f.write(f"<Scene Name=\"{name}\">\n" + "\n".join(objs) + "\n" + cam + "\n</Scene>\n")
    rad = f"<radius>{radius:.9g}</radius>" if radius is not None else ""
    cfg = (f"<Config>\n  <useGPU>0</useGPU>\n  <Scene><path>scene.xml</path><name>{name}</name><camera>cam</camera></Scene>\n"
           f"  <Renderer><type>{renderer}</type><maxDepth>{max_depth}</maxDepth>{rad}</Renderer>\n"
           f"  <time><hours>0</hours><minutes>{minutes}</minutes></time>\n</Config>\n")
    path = os.path.join(folder, "config.xml")
    with open(path, "w") as f:
        f.write(cfg)
    return path


def _read_vec(s: str):
    return tuple(float(x) for x in re.findall(r"[-+0-9.eE]+", s)[:3])


def read_obj(path: str):
    v, vn, f, fn = [], [], [], []
    with open(path) as fh:
        for line in fh:
            p = line.split()
            if not p:
                continue
            if p[0] == "v":
                v.append([float(x) for x in p[1:4]])
            elif p[0] == "vn":
                vn.append([float(x) for x in p[1:4]])
            elif p[0] == "f":
                idx = [q.split("/") for q in p[1:]]
                tri = [int(q[0]) - 1 for q in idx]
                nrm = [int(q[2]) - 1 for q in idx] if len(idx[0]) == 3 and idx[0][2] else None
                for k in range(1, len(tri) - 1):  # fan (quads split as (0,1,2),(0,2,3))
                    f.append([tri[0], tri[k], tri[k + 1]])
                    if nrm:
                        fn.append([nrm[0], nrm[k], nrm[k + 1]])
    v = np.asarray(v, np.float32)
    t = np.asarray(f, np.uint32).reshape(-1, 3)
    normals = None
    if vn and fn:
        vn = np.asarray(vn, np.float32)
        fn = np.asarray(fn, np.int64)
        if np.array_equal(fn, t.astype(np.int64)):
            normals = vn
        else:  # re-index: one normal per vertex reference
            normals = np.zeros_like(v)
            normals[t.reshape(-1)] = vn[fn.reshape(-1)]
    return v, t, normals


def read_config(path: str) -> tuple[scenes.Scene, dict]:
    """Parses a config written by write_config (or by hand in the same tag set)."""
    folder = os.path.dirname(os.path.abspath(path))
    cfg = ET.parse(path).getroot()
    sc_node = cfg.find("Scene")
    scene_file = os.path.join(folder, sc_node.findtext("path"))
    root = ET.parse(scene_file).getroot()
    objs = []
    for on in root.findall("Object"):
        mn = on.find("Material")
        kind = _KIND[mn.findtext("type").strip()]
        m = scenes.Material(kind)
        if mn.find("color") is not None:
            m.color = _read_vec(mn.findtext("color"))
        if kind == GLOSSY:
            m.coeff = float(mn.findtext("coeff"))
        if kind == REFRACTIVE:
            m.ior = float(mn.findtext("coeff") or 1.5)
            m.color = _read_vec(mn.findtext("surfColor") or "(1,1,1)")
            m.decay = _read_vec(mn.findtext("decayColor") or "(1,1,1)")
        if kind == REFLECTIVE:
            m.ior = -1.0
        if kind == PHONG:
            m.color = _read_vec(mn.find("GlossyComponent").findtext("color"))
            m.coeff = float(mn.find("GlossyComponent").findtext("coeff"))
            m.diffuse_color = _read_vec(mn.find("DiffuseComponent").findtext("color"))
        if kind == VPM:
            m.sigma_s = _read_vec(mn.findtext("sigma_s"))
            m.sigma_a = _read_vec(mn.findtext("sigma_a"))
            m.ior = float(mn.findtext("inrate"))
            m.g = float(mn.findtext("g"))
            if mn.findtext("stepsize") is not None:
                m.step_size = float(mn.findtext("stepsize"))
        v, t, n = read_obj(os.path.join(folder, on.findtext("filePath")))
        objs.append(scenes.Obj(on.get("Name", f"obj{len(objs)}"), v, t, m, n))
    cn = root.find("Camera")
    cam = scenes.Camera(int(cn.findtext("width")), int(cn.findtext("height")), int(cn.findtext("sightDist")),
                        _read_vec(cn.findtext("position")), _read_vec(cn.findtext("focus")), _read_vec(cn.findtext("up")))
    rn = cfg.find("Renderer")
    opts = {"type": rn.findtext("type"), "maxDepth": int(rn.findtext("maxDepth") or 20)}
    if rn.find("radius") is not None:
        opts["radius"] = float(rn.findtext("radius"))
    return scenes.Scene(objs, cam), opts
