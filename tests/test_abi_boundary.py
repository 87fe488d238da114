"""The C-ABI boundary on CPU: exported symbols, host-side logic, and linking
the reference's own unmodified host program against the drop-in library.

No test here launches GPU work.
"""
import ctypes as C
import os
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
INCLUDE = ROOT / "include"


@pytest.fixture(scope="module")
def libs():
    from mpifdtd_gb300 import build
    build.build()
    engine = C.CDLL(str(build.ENGINE_SO), mode=C.RTLD_GLOBAL)
    field = C.CDLL(str(build.FIELD_SO), mode=C.RTLD_GLOBAL)
    upml = C.CDLL(str(build.UPML_SO), mode=C.RTLD_GLOBAL)
    return {"engine": engine, "field": field, "upml": upml, "build": build}


def declared_functions(header: Path):
    """Function names declared in a C header (prototypes and function-pointer getters)."""
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    names = set()
    for m in re.finditer(r"\(\s*\*\s*([A-Za-z_]\w*)\s*\(\s*void\s*\)\s*\)", text):   # void (*f(void))(void)
        names.add(m.group(1))
    for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text, flags=re.M):
        if m.group(1) not in {"if", "while", "for", "return", "void", "int", "double", "char", "long"}:
            names.add(m.group(1))
    return names


def exported(so: Path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_engine_exports_every_declared_symbol(libs):
    want = declared_functions(INCLUDE / "mpifdtd_gb300.h")
    assert "fdtd_create" in want and "fdtd_ntff_step_noalloc" in want and "fdtd_spectrum" in want
    missing = want - exported(libs["build"].ENGINE_SO)
    assert not missing, missing


def test_dropin_exports_every_reference_entry_point(libs):
    want = declared_functions(INCLUDE / "mpifdtd_upml.h")
    # the four solver symbol sets of mpiTM_UPML.h, mpiTE_UPML.h, fdtdTM_upml.h, fdtdTE_upml.h
    assert len([w for w in want if w.startswith(("mpi_fdtdTM_upml_", "mpi_fdtdTE_upml_"))]) == 26
    assert len([w for w in want if w.startswith(("fdtdTM_upml_", "fdtdTE_upml_"))]) == 16
    missing = want - exported(libs["build"].UPML_SO)
    assert not missing, missing


class FieldInfo(C.Structure):  # field.h:20-28
    _fields_ = [(n, C.c_int) for n in ("width_nm", "height_nm", "h_u_nm", "pml", "lambda_nm", "angle_deg",
                                       "stepNum")]


class NTFFInfo(C.Structure):   # field.h:62-68
    _fields_ = [(n, C.c_int) for n in ("top", "bottom", "left", "right", "cx", "cy")] + \
               [("RFperC", C.c_double), ("arraySize", C.c_int)]


def test_host_field_api_matches_oracle_geometry(libs, oracle_built):
    from oracle.pyoracle import FieldInfo as OFI, OracleSim
    f = libs["field"]
    f.field_getNTFFInfo.restype = NTFFInfo
    f.field_getTime.restype = C.c_double
    f.field_getRayCoef.restype = C.c_double
    f.field_isFinish.restype = C.c_int
    for fi in [(5220, 5220, 5, 10, 500, 0, 4000), (1380, 1400, 5, 10, 400, 30, 2000), (333, 347, 3, 7, 91, 45, 10)]:
        f.field_init(FieldInfo(*fi))
        o = OracleSim("MPI_TM_UPML", OFI(*fi))
        n = f.field_getNTFFInfo()
        assert (n.top, n.bottom, n.left, n.right, n.cx, n.cy) == (o.top, o.bottom, o.left, o.right, o.cx, o.cy)
        assert n.RFperC == o.rf and n.arraySize == o.array_size
        assert C.c_int.in_dll(f, "N_PX").value == o.n_px and C.c_int.in_dll(f, "N_PY").value == o.n_py
    # clock: field.c:312-319
    f.field_init(FieldInfo(300, 320, 5, 6, 100, 0, 3))
    assert f.field_getTime() == 0 and f.field_getRayCoef() == 0
    for t in range(1, 4):
        f.field_nextStep()
        assert f.field_getTime() == t
        assert f.field_getRayCoef() == 1.0 - np.exp(-(0.01 * t) ** 2)
    assert f.field_isFinish() == 1


@pytest.mark.parametrize("model,params,oracle_model", [
    (1, [60.0, 0.0], ("circle", 60, 0.0)),
    (3, [150.0, 20.0, 25.0, 3.0, 10.0, 0.5, 0.0, 0.0], ("morpho", 150, 20, 25, 3, 10, 0.5, 0.0)),
    (5, [200.0, 50.0, 3.0, 40.0, 0.0], ("zigzag", 200, 50, 3, 40)),
])
def test_host_models_eps_equals_oracle(libs, oracle_built, model, params, oracle_model):
    """models_eps of the library's host API gives the oracle's (= reference's) permittivity bit-for-bit."""
    from oracle.pyoracle import FieldInfo as OFI, OracleSim
    from tests.golden.cases import make_model
    f = libs["field"]
    f.models_eps.restype = C.c_double
    f.models_eps.argtypes = [C.c_double, C.c_double, C.c_int]
    f.mpifdtd_models_set_params.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_int]
    fi = (330, 340, 5, 6, 90, 0, 130)
    p = (C.c_double * len(params))(*params)
    assert f.mpifdtd_models_set_params(model, p, len(params)) == 0
    f.field_init(FieldInfo(*fi))
    f.models_initModel()
    o = OracleSim("MPI_TE_UPML", OFI(*fi), make_model(oracle_model))
    want = o.eps(0)[1:-1, 1:-1]   # EPS_EX = eps(x+0.5, y, D_Y)
    got = np.array([[f.models_eps(x + 0.5, y, 1) for y in range(o.n_py)] for x in range(o.n_px)])
    np.testing.assert_array_equal(got, want)


def test_dropin_without_gpu_reports_and_returns(libs):
    """With error mode 1 a failing init() returns with the engine's status
    instead of exiting (the reference's own behaviour, exit(2), is the default)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    f, u = libs["field"], libs["upml"]
    u.mpifdtd_upml_set_error_mode(1)
    f.field_init(FieldInfo(300, 320, 5, 6, 100, 0, 10))
    f.models_setModel(0)
    f.models_initModel()
    u.mpi_fdtdTM_upml_getInit.restype = C.CFUNCTYPE(None)
    u.mpi_fdtdTM_upml_getInit()()
    assert u.mpifdtd_upml_last_status() == 2   # FDTD_E_CUDA: no device, no CPU path


REF = __import__("oracle.pyoracle", fromlist=["REF_SRC"]).REF_SRC   # $MPIFDTD_REFERENCE or ref.mk's REF
REF_HOST_SOURCES = ["main.c", "simulator.c", "field.c", "models.c", "noModel.c", "circleModel.c",
                    "morphoScaleModel.c", "multiLayerModel.c", "zigzagModel.c", "traceImageModel.c",
                    "concentricCircleModel.c", "ntffTM.c",
                    "ntffTE.c", "ntff.c", "cfft.c", "myComplex.c", "function.c", "parser.c", "drawer.c"]


@pytest.mark.skipif(not (REF / "simulator.c").exists(), reason="reference sources not present")
def test_reference_program_links_against_dropin(libs, tmp_path):
    """The reference's own host program -- main.c, simulator.c, field.c,
    models.c and the rest, unmodified -- links with libmpifdtd_upml.so in place
    of all eight solver sources (mpiTM_UPML.c, mpiTE_UPML.c, fdtdTM_upml.c,
    fdtdTE_upml.c, fdtdTM.c, fdtdTE.c, nsFdtdTM.c, nsFdtdTE.c)."""
    b = libs["build"]
    exe = tmp_path / "mpi_fdtd2D"
    cmd = ["gcc", "-std=gnu99", "-O1", "-w", "-DLINUX_OS", f"-I{ROOT / 'oracle' / 'mpi_stub'}", f"-I{REF}",
           "-o", str(exe)] + [str(REF / s) for s in REF_HOST_SOURCES] + \
          [f"-L{b.BUILD}", "-lmpifdtd_upml", "-lmpifdtd_gb300", f"-Wl,-rpath,{b.BUILD}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    syms = subprocess.run(["nm", str(exe)], capture_output=True, text=True).stdout
    assert " U mpi_fdtdTM_upml_getUpdate" in syms and " U fdtdTE_upml_getInit" in syms
    assert " U fdtdTM_getUpdate" in syms and " U nsFdtdTE_getInit" in syms


class _EngineConfig(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("width_nm", "height_nm", "h_u_nm", "pml", "lambda_nm", "angle_deg",
                                       "step_num", "precision", "flags", "courant_e4", "pml_order",
                                       "ntff_inset")] + [("reserved", C.c_int * 4)]


@pytest.mark.parametrize("courant,order,inset", [(0, 0, 0), (0.5, 3, 20), (0.6, 4, 8)])
def test_engine_geometry_with_settings_matches_oracle(libs, oracle_built, courant, order, inset):
    """fdtd_geometry_of (no GPU needed) and the oracle agree on the NTFF box,
    RFperC, arraySize and omega for the reference's settings and for a Courant
    number, grading order and NTFF inset the reference hard-codes."""
    from mpifdtd_gb300.engine import Geometry
    from oracle.pyoracle import FieldInfo as OFI, OracleSim
    e = libs["engine"]
    e.fdtd_geometry_of.argtypes = [C.POINTER(_EngineConfig), C.POINTER(Geometry)]
    fi = (600, 640, 5, 8, 150, 0, 300)
    cfg = _EngineConfig(*fi, 0, 0, round(courant * 1e4), order, inset)
    g = Geometry()
    assert e.fdtd_geometry_of(C.byref(cfg), C.byref(g)) == 0
    o = OracleSim("MPI_TM_UPML", OFI(*fi, courant=courant, pml_order=order, ntff_inset=inset))
    assert (g.ntff_top, g.ntff_bottom, g.ntff_left, g.ntff_right) == (o.top, o.bottom, o.left, o.right)
    assert g.ntff_left == 8 + (inset or 5)
    assert g.rf_per_c == o.rf and g.array_size == o.array_size
    assert g.omega_s == (courant or 0.7071) * (2 * np.pi / (150 / 5))   # field.c:107-109


def test_engine_rejects_settings_out_of_range_and_for_split_solvers(libs):
    """Courant above 1/sqrt 2, a negative grading order and any setting on the
    split-field / NS solvers are refused before any device work."""
    e = libs["engine"]
    e.fdtd_create.argtypes = [C.c_int, C.POINTER(_EngineConfig), C.POINTER(C.c_void_p)]
    e.fdtd_last_error.restype = C.c_char_p
    h = C.c_void_p()
    base = (600, 640, 5, 8, 150, 0, 300, 0, 0)
    assert e.fdtd_create(4, C.byref(_EngineConfig(*base, 7072, 0, 0)), C.byref(h)) == 1        # FDTD_E_ARG
    assert e.fdtd_create(4, C.byref(_EngineConfig(*base, 0, -1, 0)), C.byref(h)) == 1
    for solver in (0, 1, 6, 7):
        assert e.fdtd_create(solver, C.byref(_EngineConfig(*base, 5000, 0, 0)), C.byref(h)) == 5   # UNSUPPORTED
        assert b"reference's Courant number" in e.fdtd_last_error()
