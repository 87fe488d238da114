"""Capture / compare helpers for the golden vectors (test infrastructure).

Arrays are always given in the global frame: N_PX x N_PY cells, y contiguous
(for the MPI solvers the one-cell halo of the one-rank sub-domain is cropped).
NTFF accumulators are the flat [360][arraySize] blocks.
"""
from __future__ import annotations

import numpy as np

from .cases import NTFF_ROWS, NTFF_ROWS_FEW


def crop(a, mpi):
    return a[1:-1, 1:-1] if mpi else a


def sketch_vector(n, salt):
    """Fixed seeded complex vector for linear sketches.  Plain sums are useless
    here: each three-tap NTFF deposit has weights b + (a-b) - a = 0, so the sum
    of a row is rounding noise; a random projection is not."""
    rng = np.random.default_rng(20261203 + 7919 * salt + n)
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def capture(fields, eps, ntff, array_size, kind, rows="all"):
    out = {}
    for w, f in enumerate(fields):
        f = np.asarray(f, dtype=np.complex128)
        out[f"field{w}_rownorm"] = np.linalg.norm(f, axis=1)
        out[f"field{w}_rowproj"] = f @ sketch_vector(f.shape[1], 1)
        if kind == "full":
            out[f"field{w}"] = f
    if kind == "full":
        for w, e in enumerate(eps):
            out[f"eps{w}"] = np.asarray(e, dtype=np.float64)
    keep = NTFF_ROWS_FEW if rows == "few" else NTFF_ROWS
    r = sketch_vector(array_size, 2)
    for w, u in enumerate(ntff):
        block = np.asarray(u, dtype=np.complex128).reshape(360, array_size)
        out[f"ntff{w}_angleproj"] = block @ r
        out[f"ntff{w}_anglenorm"] = np.linalg.norm(block, axis=1)
        if kind == "full":
            out[f"ntff{w}_rows"] = block[keep]
    return out


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    d = np.linalg.norm(b.ravel())
    n = np.linalg.norm((a - b).ravel())
    return float(n) if d == 0 else float(n / d)


# the reference's output files (bytes), checked by their own tests
FILE_KEYS = ("elliptic_text", "image_bmp")


def compare(got: dict, ref: dict, tol: float):
    """Return {key: rel-L2 error} for every key whose error exceeds tol."""
    bad = {}
    for k, v in ref.items():
        if k.startswith("meta_") or k in FILE_KEYS:
            continue
        if k not in got:
            bad[k] = float("inf")
            continue
        if k.startswith("eps"):
            e = float(np.max(np.abs(np.asarray(got[k]) - v))) if np.size(v) else 0.0
        else:
            e = rel(got[k], v)
        if not e <= tol:
            bad[k] = e
    return bad
