"""fdtd_elliptic / fdtd_write_elliptic / fdtd_write_model_image on the GPU
engine against the reference's own files for the golden cases
(field_outputElliptic, field.c:322-343; drawer_outputImage, drawer.c:253-298)."""
import numpy as np
import pytest

from oracle import outputs
from tests.golden.cases import CASES

pytestmark = pytest.mark.gpu
GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


def _run(name):
    import mpifdtd_gb300 as m
    c = CASES[name]
    g = np.load(GOLDEN / f"{name}.npz")
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]))
    sim.set_eps(*[g[f"eps{w}"] for w in range(3)])
    sim.run(c["steps"])
    return sim, g


def _parse(text: bytes):
    rows = [line.split() for line in text.decode().splitlines()]
    return np.array([int(r[0]) for r in rows]), np.array([float(r[1]) for r in rows])


@pytest.mark.parametrize("name", sorted(n for n, c in CASES.items() if "elliptic" in c.get("extras", ())))
def test_gpu_elliptic_matches_reference_file(name, tmp_path):
    sim, g = _run(name)
    path = tmp_path / "ring.txt"
    sim.write_elliptic(path)
    got_q, got_v = _parse(path.read_bytes())
    ref_q, ref_v = _parse(g["elliptic_text"].tobytes())
    assert np.array_equal(got_q, ref_q)
    assert np.abs(got_v - ref_v).max() <= 1e-6 + 1e-12      # printed with 6 decimals
    # the unprinted values: the restatement on the engine's own final field
    w = 0 if sim.tm else 1
    ref = outputs.elliptic_ring(sim.field(w), CASES[name]["fi"][4] / CASES[name]["fi"][2])
    assert np.abs(sim.elliptic() - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("name", sorted(n for n, c in CASES.items() if "image" in c.get("extras", ())))
def test_gpu_model_image_equals_reference_file(name, tmp_path):
    sim, g = _run(name)
    path = tmp_path / "image.bmp"
    sim.write_model_image(path)
    assert path.read_bytes() == g["image_bmp"].tobytes()


def test_gpu_elliptic_ring_outside_grid_rejected():
    import mpifdtd_gb300 as m
    sim = m.Simulation("MPI_TM_UPML", m.FieldInfo(200, 200, 5, 4, 400, 0, 10))   # 1.2 lambda = 96 cells > 20
    with pytest.raises(m.FdtdError):
        sim.elliptic()
