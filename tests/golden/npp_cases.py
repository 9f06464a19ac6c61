"""Seeded probe images for the closed-library warp the reference uses
(nppiWarpAffine_32f_C1R_Ctx, NPPI_INTER_LINEAR; src/cudaMain.cu:848-875 and
:916-960).  oracle/ref/npp_probe.cpp runs NPP on these; its outputs are stored
as tests/golden/npp_warp_out.bin and pin the pixel-centre, edge and NaN rules
that the oracle's and the GB300 kernel's warps follow.

Each probe: (width, height, coeffs[2][3] float64, prefill float32, src float32 [h][w]).
"""
from __future__ import annotations

import math
import struct

import numpy as np

NAN = float("nan")


def rotation_coeffs(eangle_f32: float, nx: int, ny: int):
    """The per-angle coefficients of src/cudaMain.cu:848-855 (cos/sin of the float angle)."""
    a = float(np.cos(np.float32(eangle_f32), dtype=np.float32))
    b = float(np.sin(np.float32(eangle_f32), dtype=np.float32))
    c02 = float(np.float32((1 - a) * nx / 2 - b * ny / 2.0))
    c12 = float(np.float32(b * nx / 2.0 + (1 - a) * ny / 2.0))
    return ((a, b, c02), (-b, a, c12))


def eangle(deg: float) -> float:
    return float(np.float32(float(np.float32(deg)) * math.pi / 180.0))


def _img(rng, w, h, nan_edges=False):
    img = rng.uniform(0.5, 2.0, (h, w)).astype(np.float32)
    if nan_edges:
        img[-1, :] = np.nan
        img[:, -1] = np.nan
        img[: h // 5, : w // 6] = np.nan
    return img


def probes():
    rng = np.random.Generator(np.random.PCG64(4242))
    out = []
    ident = ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    out.append((16, 16, ident, NAN, _img(rng, 16, 16)))
    out.append((13, 17, ident, NAN, _img(rng, 13, 17)))
    out.append((16, 16, ident, 0.0, _img(rng, 16, 16, True)))
    for t in (1e-4, -1e-4, 0.25, 0.5, -0.5, 0.75, 0.999, 1.0, -1.0, 1e-7, -1e-7):
        out.append((12, 10, ((1.0, 0.0, t), (0.0, 1.0, 0.0)), NAN, _img(rng, 12, 10)))
        out.append((12, 10, ((1.0, 0.0, 0.0), (0.0, 1.0, t)), NAN, _img(rng, 12, 10)))
    out.append((12, 10, ((1.0, 0.0, 0.3), (0.0, 1.0, -0.2)), NAN, _img(rng, 12, 10, True)))
    out.append((20, 20, ((0.9, 0.1, 1.3), (-0.2, 1.1, -0.7)), NAN, _img(rng, 20, 20)))
    out.append((20, 20, ((0.9, 0.1, 1.3), (-0.2, 1.1, -0.7)), NAN, _img(rng, 20, 20, True)))
    for deg in range(0, 180, 15):
        out.append((32, 32, rotation_coeffs(eangle(deg), 32, 32), NAN, _img(rng, 32, 32, True)))
    for deg in (0, 30, 90, 165):
        # the reference passes width = Ny, height = Nx (src/cudaMain.cu:488-496) with Nx = 40, Ny = 24
        out.append((24, 40, rotation_coeffs(eangle(deg), 40, 24), NAN, _img(rng, 24, 40, True)))
    for deg in (45.0, 90.0):
        out.append((31, 31, rotation_coeffs(eangle(deg), 31, 31), NAN, _img(rng, 31, 31)))
    out.append((32, 32, rotation_coeffs(1e-3, 32, 32), NAN, _img(rng, 32, 32)))
    for deg in (15.0, 90.0):
        out.append((256, 256, rotation_coeffs(eangle(deg), 256, 256), NAN, _img(rng, 256, 256, True)))
    return out


def write_probes(path: str) -> None:
    ps = probes()
    with open(path, "wb") as f:
        f.write(b"NPPPROBE")
        f.write(struct.pack("<I", len(ps)))
        for w, h, c, prefill, img in ps:
            f.write(struct.pack("<II", w, h))
            f.write(struct.pack("<6d", *c[0], *c[1]))
            f.write(struct.pack("<f", prefill))
            f.write(np.ascontiguousarray(img, np.float32).tobytes())


def read_outputs(path: str):
    raw = np.fromfile(path, np.float32)
    outs, off = [], 0
    for w, h, *_ in probes():
        outs.append(raw[off: off + w * h].reshape(h, w))
        off += w * h
    assert off == raw.size, (off, raw.size)
    return outs
