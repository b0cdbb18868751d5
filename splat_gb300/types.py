"""Host-side record layouts shared with the C ABI (include/splat.h).

The layouts are the reference's Julia isbits layouts, so a Julia caller can
hand its own arrays across the boundary without conversion:

* ``ADRAY`` -- ``ADRay`` (src/geo.jl:60-76), 136 bytes: eight ``R3`` vectors
  (position, its wavelength / x / y partials, direction and its partials),
  ``in_medium::Bool`` at 96, ``ignore_tri::Int`` at 104, ``dest::Int`` at 112,
  ``lambda, x, y :: Float32`` at 120..131, ``status::UInt8`` at 132.
* ``FTRI`` -- ``FTri = SVector{10, R3}`` (src/geo.jl:18), 120 bytes:
  plane normal (unnormalised cross product), three vertices, three vertex
  normals, three texture coordinates ``(u, v, 0)``.  Index 1 of every
  triangle array is the all-zero sentinel triangle that is never hit.
* ``RECT_LIGHT`` -- ``RectLight`` (src/ray_generators.jl:4-11), 64 bytes.

Triangle indices crossing the boundary are the reference's 1-based indices;
a hit index of 1 means "miss" (the sentinel).
"""
from __future__ import annotations

import numpy as np

STATUS_DIFFUSE = 0
STATUS_ACTIVE = 1
STATUS_INFINITY = 2

ADRAY = np.dtype(
    {
        "names": [
            "pos", "dp_dl", "dp_dx", "dp_dy", "dir", "dd_dl", "dd_dx", "dd_dy",
            "in_medium", "ignore_tri", "dest", "lam", "x", "y", "status",
        ],
        "formats": [("<f4", (3,))] * 8 + ["u1", "<i8", "<i8", "<f4", "<f4", "<f4", "u1"],
        "offsets": [0, 12, 24, 36, 48, 60, 72, 84, 96, 104, 112, 120, 124, 128, 132],
        "itemsize": 136,
    }
)

RECT_LIGHT = np.dtype(
    {
        "names": ["center", "dir", "dim1", "dim2", "res1", "res2"],
        "formats": [("<f4", (3,))] * 4 + ["<i8", "<i8"],
        "offsets": [0, 12, 24, 36, 48, 56],
        "itemsize": 64,
    }
)

FTRI_FLOATS = 30  # 10 x R3
FTRI_BYTES = 120

# Glass index models (match SPLAT_MATERIAL_* in include/splat.h).
MATERIAL_LINEAR_REF = 0  # src/material.jl:1-9
MATERIAL_CAUCHY = 1
MATERIAL_SELLMEIER = 2

# Wavelength assignment of generated rays (SPLAT_LAMBDA_*).
LAMBDA_FIXED = 0
LAMBDA_UNIFORM = 1
LAMBDA_STRATIFIED = 2


def empty_rays(n: int) -> np.ndarray:
    return np.zeros(n, dtype=ADRAY)


def rect_light(center, direction, dim1, dim2, res1: int, res2: int) -> np.ndarray:
    rec = np.zeros((), dtype=RECT_LIGHT)
    rec["center"] = center
    rec["dir"] = direction
    rec["dim1"] = dim1
    rec["dim2"] = dim2
    rec["res1"] = res1
    rec["res2"] = res2
    return rec


def upres(n: int) -> np.ndarray:
    """Sub-sample offsets of one traced ray, src/alg_types.jl:108, binary32."""
    k = np.arange(1, n + 1, dtype=np.float32)
    nf = np.float32(n)
    return ((k / nf) - np.float32(0.5)) - (np.float32(1.0) / (np.float32(2.0) * nf))
