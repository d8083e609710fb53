"""Host-side check of the C ABI's struct layouts: every ctypes mirror in
renderx_gb300/_capi.py has the size and field offsets that a C compiler gives the
struct of the same name in include/renderx.h (a probe program compiled with gcc), and
rx_ray is the 32-byte record rays_to_array packs."""
import ctypes
import os
import shutil
import subprocess

import pytest

from renderx_gb300 import _capi

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))

MIRRORS = ["rx_object", "rx_camera", "rx_pt_options", "rx_config_info", "rx_batch_item", "rx_batch_options",
           "rx_vcm_options", "rx_bpt_options", "rx_pm_options", "rx_render_stats", "rx_guide_options",
           "rx_build_options"]


def _probe_source():
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "renderx.h"', "int main(void) {"]
    for name in MIRRORS:
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for f, _ in getattr(_capi, name)._fields_:
            lines.append(f'  printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines.append('  printf("rx_ray size %zu\\n", sizeof(rx_ray));')
    lines += ["  return 0;", "}"]
    return "\n".join(lines) + "\n"


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "probe.c", d / "probe"
    src.write_text(_probe_source())
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        struct, field, value = line.split()
        table[(struct, field)] = int(value)
    return table


@pytest.mark.parametrize("name", MIRRORS)
def test_ctypes_mirror_matches_c_layout(c_layout, name):
    cls = getattr(_capi, name)
    assert ctypes.sizeof(cls) == c_layout[(name, "size")], name
    for f, _ in cls._fields_:
        assert getattr(cls, f).offset == c_layout[(name, f)], (name, f)


def test_ray_record_is_32_bytes(c_layout):
    assert c_layout[("rx_ray", "size")] == 32
