"""Regenerate the golden vectors from the reference's own C sources.

    python tests/golden/make_golden.py [case ...]

Builds oracle/_ref/libfdtdref.so from the reference sources (oracle/ref.mk;
they must be present: $MPIFDTD_REFERENCE, else the recipe's REF), runs
every case of cases.py through the reference exactly as simulator.c drives it,
and writes tests/golden/<case>.npz.  The fixtures are committed; this script
is how they were made.
"""
from __future__ import annotations

import ctypes as C
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.pyoracle import FieldInfo, RefSim  # noqa: E402
from tests.golden.cases import CASES, make_model  # noqa: E402
from tests.golden.golden_io import capture, crop  # noqa: E402

OUT = Path(__file__).resolve().parent


def reference_elliptic(sim, field):
    """The reference's field_outputElliptic (field.c:322-343) on a global-frame
    field; returns the file's bytes."""
    lib = sim.lib
    lib.field_outputElliptic.argtypes = [C.c_char_p, C.c_void_p]
    arr = np.ascontiguousarray(field, dtype=np.complex128)
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "ring.txt"
        lib.field_outputElliptic(str(path).encode(), arr.ctypes.data)
        return np.frombuffer(path.read_bytes(), dtype=np.uint8).copy()


def reference_image(sim, eps):
    """The reference's drawer_outputImage (drawer.c:253-298) of a global-frame
    permittivity array; returns the BMP's bytes."""
    lib = sim.lib
    lib.drawer_outputImage.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    arr = np.ascontiguousarray(eps, dtype=np.float64)
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "image.bmp"
        lib.drawer_outputImage(str(path).encode(), None, arr.ctypes.data, arr.shape[0], arr.shape[1])
        return np.frombuffer(path.read_bytes(), dtype=np.uint8).copy()


def run_case(name, c):
    fi = FieldInfo(*c["fi"])
    model = make_model(c["model"])
    sim = RefSim(c["solver"], fi, model)
    sim.step(c["steps"])
    mpi = c["solver"].startswith("MPI")
    fields = [crop(sim.field(w), mpi) for w in range(3)]
    eps = [crop(sim.eps(w), mpi) for w in range(3)]
    ntff = [] if c.get("no_ntff") else [sim.ntff(w) for w in range(3)]   # split-field / NS: no NTFF
    out = capture(fields, eps, ntff, sim.array_size, c["kind"], c.get("rows", "all"))
    extras = c.get("extras", ())
    if "spectrum" in extras:
        with tempfile.TemporaryDirectory() as d:
            out["spectrum"] = sim.time_output(d)
    if "frequency" in extras:
        out["frequency"] = sim.frequency_from(*fields)
    tm = "TM" in c["solver"]
    if "elliptic" in extras:   # field_outputElliptic on Ez (TM) / Ey (TE), as the solvers call it
        out["elliptic_text"] = reference_elliptic(sim, fields[0 if tm else 1])
    if "image" in extras:      # drawer_outputImage of getEps(): EPS_EZ (TM) / EPS_EY (TE)
        out["image_bmp"] = reference_image(sim, eps[0 if tm else 1])
    out["meta_time"] = np.array(sim.time)
    out["meta_array_size"] = np.array(sim.array_size)
    return out


def main(names):
    for name in names or CASES:
        out = run_case(name, CASES[name])
        np.savez_compressed(OUT / f"{name}.npz", **out)
        print(f"{name}: {sum(v.nbytes for v in out.values()) / 1e6:.2f} MB raw")


if __name__ == "__main__":
    main(sys.argv[1:])
