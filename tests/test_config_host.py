"""CPU checks of the library's C++ scene ingest (rx_config_read: the reference's config /
scene XML and OBJ / .shp meshes, ConfigManager::load and SimpleShape::loadShape), its
PFM writer (MCRenderer::saveImagePFM) and the command-line renderer's argument handling.
No device is needed."""
import os
import subprocess

import numpy as np
import pytest

import renderx_gb300 as rx
from renderx_gb300 import build, film, scenes, sceneio

FIELDS = ("tri_begin", "tri_count", "material", "has_vertex_normals", "coeff", "ior", "g", "step_size")
VECS = ("color", "diffuse_color", "sigma_s", "sigma_a", "decay")


@pytest.mark.parametrize("name", ["cornell_box", "material_spheres", "medium_scene"])
def test_config_round_trip_is_exact(tmp_path, name):
    sc = getattr(scenes, name)(40, 30)
    cfg = sceneio.write_config(sc, str(tmp_path), "VCM" if name == "medium_scene" else "PTtest", 12, radius=0.05)
    arrays, info = rx.config_read(cfg)
    f = sc.flatten()
    assert np.array_equal(arrays["verts"], f["verts"])
    assert np.array_equal(arrays["tris"], f["tris"])
    assert np.array_equal(arrays["tri_obj"], f["tri_obj"])
    assert np.array_equal(arrays["tri_local"], f["tri_local"])
    has = np.repeat([o.normals is not None for o in sc.objects], [len(o.verts) for o in sc.objects])
    if not has.any():
        assert arrays["normals"] is None
    else:
        want_n = np.asarray(f["normals"], np.float32)[has]
        want_n = want_n / np.linalg.norm(want_n, axis=1, keepdims=True)  # loadShape normalises "vn"
        assert np.allclose(arrays["normals"][has], want_n, rtol=0, atol=2e-7)
    want = rx.objects_from_scene(sc)
    assert len(arrays["objects"]) == len(want)
    for a, b in zip(arrays["objects"], want):
        for k in FIELDS:
            if k == "coeff" and b.material not in (scenes.GLOSSY, scenes.PHONG):
                continue
            if k in ("ior", "g") and b.material not in (scenes.REFRACTIVE, scenes.REFLECTIVE, scenes.VPM):
                continue
            if k == "step_size" and b.material != scenes.VPM:
                continue
            assert getattr(a, k) == pytest.approx(getattr(b, k), rel=1e-7), (k, b.material)
        for k in VECS:
            if k == "diffuse_color" and b.material != scenes.PHONG:
                continue
            if k in ("sigma_s", "sigma_a") and b.material != scenes.VPM:
                continue
            if k == "decay" and b.material != scenes.REFRACTIVE:
                continue
            assert list(getattr(a, k)) == pytest.approx(list(getattr(b, k)), rel=1e-7), (k, b.material)
    assert info["estimator"] == (2 if name == "medium_scene" else 1)
    assert info["max_depth"] == 12
    assert info["num_triangles"] == len(f["tris"])
    c = info["camera"]
    assert (c.width, c.height, c.sight_dist) == (sc.camera.width, sc.camera.height, sc.camera.sight_dist)
    assert np.allclose(c.position, sc.camera.position) and np.allclose(c.focus, sc.camera.focus)
    if name == "medium_scene":
        assert info["radius"] == pytest.approx(0.05)


def _write(path, text):
    with open(path, "w") as fh:
        fh.write(text)


def test_quads_texcoords_transform_and_material_reference(tmp_path):
    # a unit quad (one "f" line with four v/t/n corners) and a triangle with plain indices
    _write(tmp_path / "quad.obj", "# quad\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvn 0 0 2\n"
                                  "f 1/1/1 2/1/1 3/1/1 4/1/1\n")
    _write(tmp_path / "tri.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    _write(tmp_path / "mats.xml", "<Material Name=\"red\"><type>Diffuse</type><color>(0.5, 0.1, 0.1)</color></Material>")
    _write(tmp_path / "scene.xml",
           "<Scene Name=\"s\">\n"
           "  <Material Name=\"shiny\"><type>Glossy</type><color>(0.9, 0.9, 0.9)</color><coeff>250</coeff></Material>\n"
           "  <Object Name=\"q\"><filePath>quad.obj</filePath>"
           "<transform>[1, 0, 0, 2][0, 1, 0, 3][0, 0, 1, 4][0, 0, 0, 1]</transform>"
           "<Material><path>mats.xml</path><name>red</name></Material></Object>\n"
           "  <!-- a comment -->\n"
           "  <Object Name=\"t\"><filePath>tri.obj</filePath><Material><name>shiny</name></Material></Object>\n"
           "  <Object Name=\"l\"><filePath>tri.obj</filePath><Material><type>Emissive</type>"
           "<color>(17, 12, 4)</color></Material></Object>\n"
           "  <Camera Name=\"c\"><width>8</width><height>6</height><sightDist>10</sightDist>"
           "<focus>(0, 0, 0)</focus><position>(0, 0, 5)</position><up>(0, 1, 0)</up></Camera>\n"
           "</Scene>\n")
    _write(tmp_path / "config.xml", "<?xml version=\"1.0\"?>\n<Config><Scene><path>scene.xml</path><name>s</name>"
                                    "<camera>c</camera></Scene><Renderer><type>PT</type><spp>7</spp></Renderer>"
                                    "<time><hours>1</hours><minutes>2</minutes></time>"
                                    "<savePath>out.pfm</savePath></Config>\n")
    a, info = rx.config_read(str(tmp_path / "config.xml"))
    assert a["tris"].tolist() == [[0, 1, 2], [0, 2, 3], [4, 5, 6], [7, 8, 9]]
    assert np.array_equal(a["verts"][:4], np.array([[2, 3, 4], [3, 3, 4], [3, 4, 4], [2, 4, 4]], np.float32))
    assert np.allclose(a["normals"][:4], [0, 0, 1])  # normalised on load
    o = a["objects"]
    assert [x.material for x in o] == [scenes.DIFFUSE, scenes.GLOSSY, scenes.EMISSIVE]
    assert list(o[0].color) == pytest.approx([0.5, 0.1, 0.1]) and o[1].coeff == 250
    assert [x.has_vertex_normals for x in o] == [1, 0, 0]
    assert info["estimator"] == 0 and info["spp"] == 7 and info["max_depth"] == 20
    assert info["runtime_s"] == 3720 and info["save_path"] == "out.pfm"


def _one_object(tmp_path, obj_text):
    _write(tmp_path / "m.obj", obj_text)
    _write(tmp_path / "scene.xml",
           "<Scene Name=\"s\"><Object Name=\"m\"><filePath>m.obj</filePath><Material><type>Diffuse</type>"
           "</Material></Object><Camera Name=\"c\"><width>4</width><height>4</height><sightDist>5</sightDist>"
           "<focus>(0,0,0)</focus><position>(0,0,1)</position><up>(0,1,0)</up></Camera></Scene>\n")
    _write(tmp_path / "config.xml", "<Config><Scene><path>scene.xml</path><name>s</name><camera>c</camera></Scene>"
                                    "<Renderer><type>PT</type></Renderer></Config>\n")
    return rx.config_read(str(tmp_path / "config.xml"))[0]


def test_obj_line_forms_as_sscanf_reads_them(tmp_path):
    # SimpleShape::loadShape reads lines with sscanf: a "v" needs three numbers on its own
    # line (signs, tabs and CR allowed), corners "a", "a/b", "a/" carry no normal, at most
    # four corners per face (a quad splits into (0,1,2), (0,2,3)), unknown tags are skipped
    a = _one_object(tmp_path, "# c\nv 0 0 0\nv\t1 0 0\r\nv +0 1e0 0\nv 0 0\n1\nv 1 1 0\nvt 0 0\n"
                              "usemtl x\nf 1 2 3\nf 1/9 2/ 4\r\nf 1 2 4 3 2\nf 1 2\n")
    assert a["verts"].tolist() == [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]]
    assert a["tris"].tolist() == [[0, 1, 2], [0, 1, 3], [0, 1, 3], [0, 3, 2]]
    assert a["objects"][0].has_vertex_normals == 0


def test_obj_normals_split_shared_positions(tmp_path):
    # a/b/c and a//c carry normal c (normalised); a position met again with another
    # normal becomes its own vertex
    a = _one_object(tmp_path, "v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nvn 0 0 2\nvn 0 0 -1\n"
                              "f 1/5/1 2/1/1 3/1/1\nf 1//2 2//2 4//2\n")
    assert a["tris"].tolist() == [[0, 1, 2], [4, 5, 3]]
    assert a["verts"].tolist() == [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0, 0, 0], [1, 0, 0]]
    assert a["normals"].tolist() == [[0, 0, 1]] * 3 + [[0, 0, -1]] * 3
    assert a["objects"][0].has_vertex_normals == 1


def test_shp_mesh(tmp_path):
    v = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    f = np.array([0, 1, 2], np.uint32)
    with open(tmp_path / "m.shp", "wb") as fh:
        fh.write(np.int32(9).tobytes() + v.tobytes() + np.int32(3).tobytes() + f.tobytes())
    _write(tmp_path / "config.xml",
           "<Config><Scene><name>s</name><camera>c</camera></Scene><Renderer><type>PTtest</type></Renderer></Config>\n"
           "<Scene Name=\"s\"><Object><filePath>m.shp</filePath><Material><type>Diffuse</type></Material></Object>"
           "<Camera Name=\"c\"><width>4</width><height>4</height><sightDist>5</sightDist><focus>(0,0,0)</focus>"
           "<position>(0,0,1)</position><up>(0,1,0)</up></Camera></Scene>\n")
    a, info = rx.config_read(str(tmp_path / "config.xml"))
    assert np.array_equal(a["verts"].reshape(-1), v) and a["tris"].tolist() == [[0, 1, 2]]
    assert info["estimator"] == 1


@pytest.mark.parametrize("bad,msg", [
    ("<Config></Config>", "Scene"),
    ("<Config><Scene><path>missing.xml</path><camera>c</camera></Scene></Config>", "missing.xml"),
    ("<Config><Scene><camera>c</camera></Scene></Config><Scene><GroupObject/></Scene>", "GroupObject"),
    ("<Config><Scene><camera>c</camera></Scene></Config><Scene><Object><filePath>x.obj</filePath>"
     "<Material><type>Diffuse</type><Texture/></Material></Object></Scene>", "textured"),
    ("<Config><Scene><camera>c</camera>", "unterminated"),
])
def test_config_errors(tmp_path, bad, msg):
    _write(tmp_path / "config.xml", bad)
    with pytest.raises(rx.RxError, match=msg):
        rx.config_read(str(tmp_path / "config.xml"))


def test_pfm_writer_matches_reference_layout(tmp_path):
    img = np.arange(2 * 3 * 3, dtype=np.float64).reshape(2, 3, 3) / 7.0
    p = str(tmp_path / "a.pfm")
    rx.write_pfm(p, img)
    raw = open(p, "rb").read()
    assert raw.startswith(b"PF\n3 2\n-1.000000\n")
    body = np.frombuffer(raw[len(b"PF\n3 2\n-1.000000\n"):], "<f4").reshape(2, 3, 3)
    assert np.array_equal(body, img[::-1].astype(np.float32))  # bottom row first, RGB
    assert np.array_equal(film.load_pfm(p), img.astype(np.float32))


def test_cli_usage():
    build.build()
    r = subprocess.run([build.CLI, "--help"], capture_output=True, text=True)
    assert r.returncode == 2 and "config.xml" in r.stderr
    r = subprocess.run([build.CLI, "x.xml", "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "unknown option" in r.stderr


@pytest.mark.parametrize("type_name,code", [("PathTracer", 0), ("PT", 0), ("PTtest", 1), ("VCMTracer", 2), ("VCM", 2),
                                            ("BidirectionalPathTracer", 3), ("BPT", 3), ("PhotonMap", 4), ("PM", 4),
                                            ("IPT", -1)])
def test_renderer_type_names(tmp_path, type_name, code):
    # ConfigManager.cpp:323-354: the <Renderer><type> names and the renderer each selects
    sc = scenes.cornell_box(8, 8)
    cfg = sceneio.write_config(sc, str(tmp_path), type_name, 5)
    _, info = rx.config_read(cfg)
    assert info["estimator"] == code and info["renderer"] == type_name and info["max_depth"] == 5


def test_group_object_splits_unitizes_and_transforms(tmp_path):
    # ConfigManager.cpp:193-224 + SimpleShape::loadShape(path, true, &shapes): "g" lines
    # start shapes whose indices are the file's minus the vertices before the group; the
    # whole file is unitized (centre 0, largest extent 2); quads stay with the file; the
    # group's transform applies to every shape
    _write(tmp_path / "grp.obj", "v 9 9 9\n"               # before any group: counts for the box only
                                 "g left\nv 0 0 0\nv 2 0 0\nv 0 2 0\nf 2 3 4\n"
                                 "g right\nv 2 2 0\nv 4 2 0\nv 2 4 0\nv 4 4 0\nf 5 6 7\nf 5 6 8 7\n")
    _write(tmp_path / "scene.xml",
           "<Scene Name=\"s\">\n"
           "  <GroupObject><filePath>grp.obj</filePath>"
           "<transform>[1, 0, 0, 10][0, 1, 0, 0][0, 0, 1, 0][0, 0, 0, 1]</transform>"
           "<Object Name=\"right\"><Material><type>Diffuse</type><color>(0.5, 0.5, 0.5)</color></Material></Object>"
           "<Object Name=\"left\"><Material><type>Emissive</type><color>(1, 1, 1)</color></Material></Object>"
           "</GroupObject>\n"
           "  <Object Name=\"t\"><filePath>tri.obj</filePath><Material><type>Diffuse</type></Material></Object>\n"
           "  <Camera Name=\"c\"><width>4</width><height>4</height><sightDist>5</sightDist><focus>(0,0,0)</focus>"
           "<position>(0,0,1)</position><up>(0,1,0)</up></Camera>\n</Scene>\n")
    _write(tmp_path / "tri.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    _write(tmp_path / "config.xml", "<Config><Scene><path>scene.xml</path><name>s</name><camera>c</camera></Scene>"
                                    "<Renderer><type>PT</type></Renderer></Config>\n")
    a, info = rx.config_read(str(tmp_path / "config.xml"))
    o = a["objects"]
    assert [x.material for x in o] == [scenes.DIFFUSE, scenes.EMISSIVE, scenes.DIFFUSE]  # group first, in order
    assert [x.tri_count for x in o] == [1, 1, 1]  # the quad of "right" is not in the shape
    # file box: (0,0,0)-(9,9,9): centre 4.5, largest extent 9 -> scale 2/9
    s, c = np.float32(2) / np.float32(9), np.float32(4.5)
    t = np.float32(-2) / np.float32(9) * c

    def unit(v):
        return np.array([s * np.float32(x) + t for x in v], np.float32) + np.array([10, 0, 0], np.float32)
    right = a["verts"][a["tris"][o[0].tri_begin]]
    left = a["verts"][a["tris"][o[1].tri_begin]]
    assert np.allclose(right, [unit(v) for v in ([2, 2, 0], [4, 2, 0], [2, 4, 0])], atol=1e-6)
    assert np.allclose(left, [unit(v) for v in ([0, 0, 0], [2, 0, 0], [0, 2, 0])], atol=1e-6)
    assert info["num_triangles"] == 3
