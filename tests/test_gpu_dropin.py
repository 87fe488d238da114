"""GPU: the drop-in solver library driven exactly as simulator.c drives a solver.

simulator_init (simulator.c:258-266): field_init, models_initModel, init();
simulator_calc (simulator.c:247-251): update(), field_nextStep(); the host
program's field.c/models.c role is played by the library's own host API
(libmpifdtd_field.so).  Results are checked against the reference's golden
vectors at 1e-12 relative L2.
"""
import ctypes as C
import os

import numpy as np
import pytest

from tests.golden.cases import CASES
from tests.golden.golden_io import rel

pytestmark = pytest.mark.gpu

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


class FieldInfo(C.Structure):  # field.h:20-28
    _fields_ = [(n, C.c_int) for n in ("width_nm", "height_nm", "h_u_nm", "pml", "lambda_nm", "angle_deg",
                                       "stepNum")]


@pytest.fixture(scope="module")
def libs():
    from mpifdtd_gb300 import build
    build.build()
    C.CDLL(str(build.ENGINE_SO), mode=C.RTLD_GLOBAL)
    field = C.CDLL(str(build.FIELD_SO), mode=C.RTLD_GLOBAL)
    upml = C.CDLL(str(build.UPML_SO), mode=C.RTLD_GLOBAL)
    field.field_isFinish.restype = C.c_int
    field.mpifdtd_models_set_params.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_int]
    return field, upml


VOIDFN = C.CFUNCTYPE(None)
PREFIX = {"MPI_TM_UPML": "mpi_fdtdTM_upml_", "MPI_TE_UPML": "mpi_fdtdTE_upml_",
          "TM_UPML": "fdtdTM_upml_", "TE_UPML": "fdtdTE_upml_",
          "TM_2D": "fdtdTM_", "TE_2D": "fdtdTE_", "NS_TM_2D": "nsFdtdTM_", "NS_TE_2D": "nsFdtdTE_"}


def _fn(lib, name, restype):
    f = getattr(lib, name)
    f.restype = restype
    f.argtypes = []
    return f


def drive(libs, name):
    """Run a golden case through the drop-in entry points; returns (upml, prefix, nx, ny)."""
    field, upml = libs
    c = CASES[name]
    kind, radius, eps = c["model"]
    assert kind == "circle"
    p = (C.c_double * 2)(radius, eps)
    assert field.mpifdtd_models_set_params(1, p, 2) == 0
    field.models_setModel(1)                                   # MIE_CYLINDER
    field.field_init(FieldInfo(*c["fi"]))
    field.models_initModel()
    pre = PREFIX[c["solver"]]
    init = _fn(upml, pre + "getInit", VOIDFN)()
    update = _fn(upml, pre + "getUpdate", VOIDFN)()
    init()
    assert upml.mpifdtd_upml_last_status() == 0
    steps = 0
    while not field.field_isFinish():                          # main.c:186-188
        update()
        field.field_nextStep()
        steps += 1
    assert steps == c["steps"]
    n_px, n_py = c["fi"][0] // c["fi"][2], c["fi"][1] // c["fi"][2]
    mpi = c["solver"].startswith("MPI")
    return upml, pre, (n_px + 2, n_py + 2) if mpi else (n_px, n_py), mpi


def _array(ptr, shape, dtype):
    n = shape[0] * shape[1] * (2 if dtype == np.complex128 else 1)
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_double)), shape=(n,)).view(dtype).reshape(shape).copy()


@pytest.mark.parametrize("name", ["mpi_tm_circle", "mpi_te_circle"])
def test_dropin_mpi_solver_matches_golden(libs, name):
    upml, pre, shape, mpi = drive(libs, name)
    ref = np.load(GOLDEN / f"{name}.npz")
    names = ("getEz", "getHx", "getHy") if "TM" in pre else ("getEx", "getEy", "getHz")
    for w, g in enumerate(names):
        a = _array(_fn(upml, pre + g, C.c_void_p)(), shape, np.complex128)
        assert np.all(a[0] == 0) and np.all(a[-1] == 0) and np.all(a[:, 0] == 0) and np.all(a[:, -1] == 0)
        assert rel(a[1:-1, 1:-1], ref[f"field{w}"]) <= 1e-12, (name, g)
    eps = _array(_fn(upml, pre + "getEps", C.c_void_p)(), shape, np.float64)
    want = ref["eps0"] if "TM" in pre else ref["eps1"]     # EPS_EZ / EPS_EY (mpiTE_UPML.c:104-106)
    np.testing.assert_array_equal(eps[1:-1, 1:-1], want)
    assert _fn(upml, pre + "getSubNpx", C.c_int)() == shape[0]
    assert _fn(upml, pre + "getSubNcell", C.c_int)() == shape[0] * shape[1]
    _fn(upml, pre + "getFinish", VOIDFN)()()
    assert upml.mpifdtd_upml_last_status() == 0


@pytest.mark.parametrize("name", ["ser_tm_circle", "ser_te_circle"])
def test_dropin_serial_reset_writes_reference_spectrum(libs, name, tmp_path):
    """reset() of the serial solvers writes the spectrum files of
    ntffTM_TimeOutput (ntffTM.c:239-247) in the working directory."""
    upml, pre, shape, _ = drive(libs, name)
    ref = np.load(GOLDEN / f"{name}.npz")
    a = _array(_fn(upml, pre + ("getEz" if "TM" in pre else "getEx"), C.c_void_p)(), shape, np.complex128)
    assert rel(a, ref["field0"]) <= 1e-12
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        _fn(upml, pre + "getReset", VOIDFN)()()
    finally:
        os.chdir(cwd)
    ang = CASES[name]["fi"][5]
    spec = np.fromfile(tmp_path / f"{ang}[deg]_380nm_700nm_b.dat", dtype=np.float64).reshape(321, 360)
    assert rel(spec, ref["spectrum"]) <= 1e-12
    txt = (tmp_path / f"{ang}[deg].txt").read_text().splitlines()
    assert len(txt) == 321 and txt[0].startswith("380 ")
    a = _array(_fn(upml, pre + ("getEz" if "TM" in pre else "getEx"), C.c_void_p)(), shape, np.complex128)
    assert np.all(a == 0)                                   # reset zeroes the fields
    os.chdir(tmp_path)
    try:
        _fn(upml, pre + "getFinish", VOIDFN)()()            # finish() writes the spectrum again (reset first)
    finally:
        os.chdir(cwd)


@pytest.mark.parametrize("name,ring", [("split_tm_circle", "tm_5nm.txt"), ("split_te_circle_30deg", "te_5nm.txt"),
                                       ("ns_te_circle_20deg", "ns_te_5nm.txt")])
def test_dropin_split_and_ns_solvers(libs, name, ring, tmp_path):
    """The split-field PML and NS-FDTD entry points (fdtdTM.h, fdtdTE.h,
    nsFdtdTE.h): fields, split parts and getEps against the reference's golden
    vectors; reset() writes field_outputElliptic's ring file."""
    upml, pre, shape, _ = drive(libs, name)
    ref = np.load(GOLDEN / f"{name}.npz")
    tm = "TM" in pre
    names = ("getEz", "getHx", "getHy") if tm else ("getEx", "getEy", "getHz")
    got = [_array(_fn(upml, pre + g, C.c_void_p)(), shape, np.complex128) for g in names]
    for w in range(3):
        assert rel(got[w], ref[f"field{w}"]) <= 1e-12, (name, names[w])
    parts = ("getEzx", "getEzy") if tm else ("getHzx", "getHzy")
    a, b = (_array(_fn(upml, pre + g, C.c_void_p)(), shape, np.complex128) for g in parts)
    if not tm:                                              # Hz = Hzx + Hzy after calcH
        np.testing.assert_array_equal(a + b, got[2])
    eps = _array(_fn(upml, pre + "getEps", C.c_void_p)(), shape, np.float64)
    np.testing.assert_array_equal(eps, ref["eps0"] if tm else ref["eps1"])   # EPS_EZ / EPS_EY
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        _fn(upml, pre + "getReset", VOIDFN)()()
    finally:
        os.chdir(cwd)
    lines = (tmp_path / ring).read_text().splitlines()
    want = ref["elliptic_text"].tobytes().decode().splitlines()
    assert len(lines) == len(want) == 181
    got_v = np.array([float(x.split()[1]) for x in lines])
    want_v = np.array([float(x.split()[1]) for x in want])
    assert np.abs(got_v - want_v).max() <= 1e-6 + 1e-12
    a = _array(_fn(upml, pre + names[0], C.c_void_p)(), shape, np.complex128)
    assert np.all(a == 0)                                   # reset zeroes the fields
    os.chdir(tmp_path)
    try:
        _fn(upml, pre + "getFinish", VOIDFN)()()            # finish() = reset() + free (writes the ring again)
    finally:
        os.chdir(cwd)
    assert upml.mpifdtd_upml_last_status() == 0
