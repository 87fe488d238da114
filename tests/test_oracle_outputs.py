"""The oracle's restatement of the reference's plain-file outputs
(oracle/outputs.py) against the files the reference itself wrote for the
golden cases: field_outputElliptic (field.c:322-343) on the final E field and
drawer_outputImage (drawer.c:253-298) of the solver's permittivity, byte for
byte."""
import numpy as np
import pytest

from oracle import outputs
from tests.golden.cases import CASES

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


def _cases(extra):
    return sorted(n for n, c in CASES.items() if extra in c.get("extras", ()))


@pytest.mark.parametrize("name", _cases("elliptic"))
def test_elliptic_restatement_equals_reference_file(name):
    c = CASES[name]
    g = np.load(GOLDEN / f"{name}.npz")
    fi = c["fi"]
    field = g["field0" if "TM" in c["solver"] else "field1"]
    vals = outputs.elliptic_ring(field, fi[4] / fi[2])
    assert outputs.elliptic_text(vals) == g["elliptic_text"].tobytes()


@pytest.mark.parametrize("name", _cases("image"))
def test_model_image_restatement_equals_reference_file(name):
    c = CASES[name]
    g = np.load(GOLDEN / f"{name}.npz")
    eps = g["eps0" if "TM" in c["solver"] else "eps1"]
    data = outputs.model_bmp(eps)
    assert data == g["image_bmp"].tobytes()
    assert data[:2] == b"BM" and len(data) == 54 + 3 * ((eps.shape[0] >> 2) << 2) * eps.shape[1]
