"""Film output and image metrics.

* ``save_pfm`` / ``load_pfm`` — MCRenderer::saveImagePFM's format (reference
  src/MCRenderer.cpp:556-574): ``PF`` header, little-endian (scale -1.0), rows stored
  bottom-up, RGB float32. The reference writes from an OpenCV BGR image and swaps
  channels back, so the file holds RGB; ``film`` here is rows-from-the-top RGB, the
  order of renderPixels' vector<vec3f>.
* ``rmse`` — cmp/compare.cpp's CalculateRMSE (:83-124): sqrt of the mean over pixels of
  the squared RGB distance (without the [0,4] clamp of visualizeUtils.h's reader).
* ``relmse`` — mean over pixels and channels of (I-R)^2 / (R^2 + 1e-2).
* ``save_png`` — 8-bit tone-mapped preview (gamma 2.2), no third-party imaging.
* ``convergence`` / ``write_convergence`` / ``load_mask`` — cmp/compare.cpp's
  calcRMSEs (:242-331): every ``*_time_<t>_iter_<s>.pfm`` snapshot (the names
  MCRenderer::showCurrentResult writes, src/MCRenderer.cpp:465-490) against a reference
  image, optionally inside a mask (whitespace-separated 0/1 per pixel, rows from the
  bottom), sorted by time and written as ``time rmse`` lines.
"""
from __future__ import annotations

import glob
import os
import struct
import zlib

import numpy as np


def save_pfm(path: str, film: np.ndarray):
    img = np.asarray(film, np.float32)
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.000000\n".encode())
        f.write(np.ascontiguousarray(img[::-1]).astype("<f4").tobytes())


def load_pfm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        if f.readline().strip() != b"PF":
            raise ValueError("not an RGB PFM")
        w, h = (int(x) for x in f.readline().split())
        scale = float(f.readline())
        dt = "<f4" if scale < 0 else ">f4"
        data = np.frombuffer(f.read(w * h * 12), dt).reshape(h, w, 3)
    return data[::-1].astype(np.float32)


def rmse(img: np.ndarray, ref: np.ndarray, mask: np.ndarray | None = None) -> float:
    d = np.sum((np.asarray(img, np.float64) - np.asarray(ref, np.float64)) ** 2, axis=-1)
    if mask is not None:
        d = d[mask]
    return float(np.sqrt(d.mean()))


def relmse(img: np.ndarray, ref: np.ndarray) -> float:
    i = np.asarray(img, np.float64)
    r = np.asarray(ref, np.float64)
    return float(np.mean((i - r) ** 2 / (r * r + 1e-2)))


def save_png(path: str, film: np.ndarray, exposure: float = 1.0):
    img = np.clip(np.asarray(film, np.float64) * exposure, 0, 1) ** (1 / 2.2)
    a = (img * 255 + 0.5).astype(np.uint8)
    h, w, _ = a.shape
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))

    def chunk(t, d):
        c = struct.pack(">I", len(d)) + t + d
        return c + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
                + chunk(b"IDAT", zlib.compress(raw, 9)) + chunk(b"IEND", b""))


def snapshot_stamp(name: str):
    """(time, iter) of a snapshot file name, or None: the tokens between '_' and '.'
    that follow "time" and "iter" (compare.cpp's parser)."""
    time = it = None
    toks = name.replace(".", "_").split("_")
    for a, b in zip(toks, toks[1:]):
        if a == "time" and b.lstrip("-").isdigit():
            time = int(b)
        if a == "iter" and b.lstrip("-").isdigit():
            it = int(b)
    return None if time is None or it is None else (time, it)


def load_mask(path: str, width: int, height: int) -> np.ndarray:
    """compare.cpp's mask file: width*height integers, rows from the bottom; True = 1."""
    vals = np.array(open(path).read().split(), np.int64)[: width * height]
    return (vals.reshape(height, width) == 1)[::-1]


def convergence(paths, ref: np.ndarray, mask: np.ndarray | None = None):
    """[(time, iter, rmse, relmse)] of the stamped snapshots among ``paths`` (a list of
    files or one directory), sorted by time."""
    if isinstance(paths, str):
        paths = sorted(glob.glob(os.path.join(paths, "*.pfm")))
    rows = []
    for p in paths:
        st = snapshot_stamp(os.path.basename(p))
        if st is None:
            continue
        img = load_pfm(p)
        rows.append((st[0], st[1], rmse(img, ref, mask), relmse(img, ref)))
    rows.sort(key=lambda r: r[0])
    return rows


def write_convergence(path: str, rows):
    """compare.cpp's output: one "time rmse" line per snapshot."""
    with open(path, "w") as f:
        for t, _, e, _ in rows:
            f.write(f"{t} {e:.8f}\n")
