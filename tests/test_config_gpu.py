"""GPU checks of the config-file path: a scene read by the library's C++ loader renders
the same image as the same scene uploaded from Python, and the command-line renderer
renders a config end to end into a PFM."""
import os
import subprocess

import numpy as np
import pytest

import renderx_gb300 as rx
from renderx_gb300 import build, film, scenes, sceneio

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,nee", [("material_spheres", True), ("medium_scene", False)])
def test_loaded_config_renders_like_python_upload(tmp_path, name, nee):
    sc = getattr(scenes, name)(32, 24)
    cfg = sceneio.write_config(sc, str(tmp_path), "PTtest" if nee else "PT", 8)
    with rx.Context(0) as a, rx.Context(0) as b:
        info = a.load_config(cfg)
        a.build_accel()
        b.set_scene(sc)
        b.build_accel()
        ia, _, _ = a.render_pt(info["camera"], 64, max_depth=info["max_depth"], nee=nee, seed=5)
        ib, _, _ = b.render_pt(sc.camera, 64, max_depth=8, nee=nee, seed=5)
    assert info["estimator"] == (1 if nee else 0)
    # same geometry bit for bit (vertex normals are normalised on load, as SimpleShape does)
    assert np.allclose(ia, ib, rtol=1e-4, atol=1e-6)


def test_cli_renders_config(tmp_path):
    sc = scenes.cornell_box(32, 32)
    cfg = sceneio.write_config(sc, str(tmp_path), "PT", 8)
    build.build()
    out = str(tmp_path / "img.pfm")
    r = subprocess.run([build.CLI, cfg, "--spp", "256", "--out", out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    img = film.load_pfm(out)
    with rx.Context(0) as c:
        c.set_scene(sc)
        c.build_accel()
        ref, _, _ = c.render_pt(sc.camera, 256, max_depth=8, seed=1)
    assert img.shape == (32, 32, 3)
    assert np.allclose(img, ref.astype(np.float32), rtol=1e-4, atol=1e-6)
    # VCM through the same front end
    cfg2 = sceneio.write_config(sc, str(tmp_path / "v"), "VCM", 8, radius=0.05)
    r = subprocess.run([build.CLI, cfg2, "--iterations", "2", "--out", str(tmp_path / "v.pfm")], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert np.isfinite(film.load_pfm(str(tmp_path / "v.pfm"))).all()
    # BidirectionalPathTracer and PhotonMap through the same front end, equal to the API's renders
    for typ, args, fn in (("BPT", ["--spp", "4"], lambda c: c.render_bpt(sc.camera, 4, max_depth=8, seed=1)[0]),
                          ("PM", ["--iterations", "2"],
                           lambda c: c.render_pm(sc.camera, 2, 0.05, max_depth=8, seed=1)[0])):
        d = tmp_path / typ
        cfg3 = sceneio.write_config(sc, str(d), typ, 8, radius=0.05)
        r = subprocess.run([build.CLI, cfg3, *args, "--out", str(d / "img.pfm")], capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr
        img3 = film.load_pfm(str(d / "img.pfm"))
        with rx.Context(0) as c:
            c.set_scene(sc)
            c.build_accel()
            want = fn(c)
        assert img3.mean() > 0
        assert np.allclose(img3, want.astype(np.float32), rtol=2e-3, atol=1e-5), typ


def test_cli_writes_time_stamped_snapshots(tmp_path):
    # MCRenderer::showCurrentResult's names <stem>_time_<t>_iter_<s>.pfm, read back by
    # the convergence tooling; the last snapshot is the final image
    sc = scenes.cornell_box(32, 32)
    cfg = sceneio.write_config(sc, str(tmp_path), "PT", 8)
    build.build()
    out = str(tmp_path / "img.pfm")
    r = subprocess.run([build.CLI, cfg, "--spp", "3", "--snapshot-every", "0.000001", "--out", out],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rows = film.convergence(str(tmp_path), film.load_pfm(out))
    assert sorted(it for _, it, _, _ in rows)[-1] == 2
    assert rows[-1][2] < 1e-6  # the last snapshot holds all three samples
