"""Host-side checks of the film tooling: the PFM round trip, and the convergence table
of time-stamped snapshots (cmp/compare.cpp's calcRMSEs: names *_time_<t>_iter_<s>.pfm,
RMSE against a reference inside an optional bottom-up 0/1 mask, sorted by time, written
as "time rmse" lines)."""
import numpy as np

from renderx_gb300 import film


def test_snapshot_stamp_parses_reference_names():
    assert film.snapshot_stamp("cb_time_300_iter_41.pfm") == (300, 41)
    assert film.snapshot_stamp("a_b_iter_7_time_12.pfm") == (12, 7)
    assert film.snapshot_stamp("result.pfm") is None
    assert film.snapshot_stamp("x_time_5.pfm") is None


def test_convergence_table_sorted_by_time_with_mask(tmp_path):
    rng = np.random.default_rng(3)
    ref = rng.random((6, 5, 3)).astype(np.float32)
    film.save_pfm(str(tmp_path / "ref_unstamped.pfm"), ref)
    errs = {}
    for t, it, noise in ((600, 80, 0.05), (300, 40, 0.1), (900, 120, 0.02)):
        img = (ref + noise * rng.standard_normal(ref.shape)).astype(np.float32)
        film.save_pfm(str(tmp_path / f"cb_time_{t}_iter_{it}.pfm"), img)
        errs[t] = img
    rows = film.convergence(str(tmp_path), ref)
    assert [r[0] for r in rows] == [300, 600, 900] and [r[1] for r in rows] == [40, 80, 120]
    for t, it, e, rel in rows:
        d = np.sum((errs[t].astype(np.float64) - ref) ** 2, axis=-1)
        assert np.isclose(e, np.sqrt(d.mean()))
        assert np.isclose(rel, film.relmse(errs[t], ref))
    # mask file: rows from the bottom, 1 = inside
    m = np.zeros((6, 5), bool)
    m[0, :] = True  # top row
    (tmp_path / "mask.txt").write_text(" ".join(str(int(v)) for v in m[::-1].ravel()))
    mask = film.load_mask(str(tmp_path / "mask.txt"), 5, 6)
    assert np.array_equal(mask, m)
    rows_m = film.convergence(str(tmp_path), ref, mask)
    d = np.sum((errs[300].astype(np.float64) - ref) ** 2, axis=-1)
    assert np.isclose(rows_m[0][2], np.sqrt(d[m].mean()))
    film.write_convergence(str(tmp_path / "rmse.txt"), rows)
    lines = (tmp_path / "rmse.txt").read_text().splitlines()
    assert [ln.split()[0] for ln in lines] == ["300", "600", "900"]
    assert float(lines[0].split()[1]) == float(f"{rows[0][2]:.8f}")


def test_pfm_round_trip(tmp_path):
    img = np.random.default_rng(1).random((4, 7, 3)).astype(np.float32)
    film.save_pfm(str(tmp_path / "a.pfm"), img)
    assert np.array_equal(film.load_pfm(str(tmp_path / "a.pfm")), img)
