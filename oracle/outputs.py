"""Restatement of the reference's two plain-file outputs besides the spectrum.

TEST INFRASTRUCTURE (the oracle).  Checks fdtd_write_elliptic and
fdtd_write_model_image; the product never imports it.

  elliptic_ring  field_outputElliptic (field.c:322-343) with cbilinear and
                 cnorm (myComplex.c:33-52)
  model_bmp      drawer_outputImage (drawer.c:253-298) with colorTransform /
                 modelColorTransform (drawer.c:230-251), putBmpHeader and its
                 little-endian byte writers (drawer.c:312-445)
"""
from __future__ import annotations

import math
import struct

import numpy as np


def elliptic_ring(field: np.ndarray, lambda_s: float) -> np.ndarray:
    """|field|^2 on the 1.2 lambda_s circle, 181 values, index q = 180 - ang.

    field: global frame N_PX x N_PY complex (y contiguous)."""
    n_px, n_py = field.shape
    flat = np.ascontiguousarray(field, dtype=np.complex128).reshape(-1)
    out = np.empty(181)
    for ang in range(180, -1, -1):
        rad = ang * math.pi / 180.0
        x = 1.2 * lambda_s * math.cos(rad) + n_px / 2.0
        y = 1.2 * lambda_s * math.sin(rad) + n_py / 2.0
        i, j = math.floor(x), math.floor(y)
        dx, dy = x - i, y - j
        k = i * n_py + j
        p0, p1, p2, p3 = flat[k], flat[k + n_py], flat[k + 1], flat[k + n_py + 1]
        re = p0.real * (1.0 - dx) * (1.0 - dy) + p1.real * dx * (1.0 - dy) + p2.real * (1.0 - dx) * dy + p3.real * dx * dy
        im = p0.imag * (1.0 - dx) * (1.0 - dy) + p1.imag * dx * (1.0 - dy) + p2.imag * (1.0 - dx) * dy + p3.imag * dx * dy
        out[180 - ang] = re * re + im * im
    return out


def elliptic_text(values: np.ndarray) -> bytes:
    """The file field_outputElliptic writes: "%d %lf \\n" per line."""
    return "".join("%d %f \n" % (q, v) for q, v in enumerate(values)).encode()


def _channel(v: np.float32) -> int:
    x = np.float32(v) * np.float32(255)
    m = np.float32(255) if np.float32(255) < x else x
    return int(np.float32(0) if np.float32(0) > m else m)


def model_bmp(eps: np.ndarray) -> bytes:
    """24-bit BMP bytes of a global-frame permittivity array (N_PX x N_PY)."""
    width, height = eps.shape
    data_width = (width >> 2) << 2
    head = b"BM" + struct.pack("<IHHIIiiHHIIiiII", 54 + data_width * height, 0, 0, 54, 40,
                               data_width, height, 1, 24, 0, 0, 0, 0, 0, 0)
    pix = bytearray()
    lut = {}
    for j in range(height):
        for i in range(data_width):
            n = float(eps[i, j])
            c = lut.get(n)
            if c is None:
                d = 1 - 1.0 / n / n
                r = np.float32(0.0 - d)
                g = np.float32(1.0 - d)
                c = lut[n] = bytes((_channel(r), _channel(g), _channel(r)))   # b, g, r; b == r
            pix += c
    return head + bytes(pix)
