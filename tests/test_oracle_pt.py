"""Pins the path-tracing oracle: the CPU restatement of the reference's PathTracer
(oracle/rxo_pt.cpp, over the restated reference tree) agrees per pixel with the
reference's own renders (tests/golden/render_*_pt.npz, made by the reference's
PathTracer compiled from its sources) within 3 sigma of the combined standard error:
at most 1% of channels beyond 3 sigma, none beyond 6, no signed bias over the crop.
Both sides render 4096 samples (comparable noise: the estimator is heavy-tailed, so a
pixel's sample variance underestimates its error where its mean falls short)."""
import os

import numpy as np
import pytest

import oracle
from renderx_gb300 import scenes


@pytest.mark.parametrize("name,crop,spp", [("cornell_pt", (16, 16, 32, 32), 4096),
                                           ("spheres_pt", (14, 30, 36, 20), 4096)])
def test_pt_oracle_matches_reference_renders(name, crop, spp):
    z = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", f"render_{name}.npz")))
    assert str(z["mode"]) == "pt"
    sc = getattr(scenes, str(z["scene"]))(64, 64)
    x0, y0, w, h = crop
    m, sq, rays = oracle.RefPathTracer(sc).render(sc.camera, spp, max_depth=int(z["max_depth"]), rr_mode=0, seed=5,
                                                  crop=crop, want_sq=True)
    assert rays > w * h * spp  # camera rays and bounces
    se = np.sqrt(np.maximum(sq - m * m, 0.0) / (spp - 1))
    ref = z["mean"][y0:y0 + h, x0:x0 + w].astype(np.float64)
    rse = z["stderr"][y0:y0 + h, x0:x0 + w].astype(np.float64)
    zz = (m - ref) / np.sqrt(se ** 2 + rse ** 2 + 1e-30)
    assert (np.abs(zz) > 3).mean() <= 0.01, f"{(np.abs(zz) > 3).mean():.4f} beyond 3 sigma"
    assert np.abs(zz).max() < 6
    assert np.all(np.abs(zz.mean(axis=(0, 1))) < 4 / np.sqrt(w * h))  # no signed bias
