"""Host-side checks of the library (no GPU): the reference-order tree the library
builds equals the reference's serialized tree, and the C ABI exports every entry point
declared in include/renderx.h."""
import os
import re

import numpy as np
import pytest

import oracle
import renderx_gb300 as rx
from renderx_gb300 import _capi
from golden_util import CASES, load

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


@pytest.mark.parametrize("name", CASES)
def test_library_reftree_equals_reference(name):
    z = load(name)
    nodes, leaf = rx.reftree_serialize(z["verts"], z["tris"], rx.SPLIT_GCC)
    assert np.array_equal(nodes, z["nodes"])
    assert np.array_equal(leaf, z["leaf"])


@pytest.mark.parametrize("name", ["cornell", "spheres4"])
def test_library_reftree_best_axis_policy_equals_oracle(name):
    z = load(name)
    a = oracle.RefTree(z["verts"], z["tris"], oracle.SPLIT_BEST).serialize()
    b = rx.reftree_serialize(z["verts"], z["tris"], rx.SPLIT_BEST)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_reftree_rejects_bad_input():
    v = np.zeros((3, 3), np.float32)
    t = np.array([[0, 1, 5]], np.uint32)
    with pytest.raises(rx.RxError):
        rx.reftree_serialize(v, t)


def _header_functions():
    src = open(os.path.join(ROOT, "include", "renderx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rx_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    names = _header_functions()
    assert len(names) >= 10
    L = _capi.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    bound = {s[0] for s in _capi.SIGNATURES}
    assert set(names) <= bound, set(names) - bound


def test_version_string():
    assert b"sm_103a" in _capi.lib().rx_version()
