"""Python access to the two CPU oracles.  TEST INFRASTRUCTURE.

* ``OracleSim`` wraps ``fdtd_oracle.c``, the project's C restatement of the
  reference's UPML path (built into ``oracle/_build``).  It runs anywhere a C
  compiler exists and is what the tests compare the CUDA path with, and the
  CPU baseline of ``bench.py``.
* ``RefSim`` wraps the reference's own C sources compiled unmodified
  (``oracle/ref.mk`` -> ``oracle/_ref/libfdtdref.so``).  It exists only where
  the reference sources are present and pins ``OracleSim``; its outputs are
  frozen into ``tests/golden`` by ``tests/golden/make_golden.py``.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  The product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "libfdtd_oracle.so"
REF_SO = HERE / "_ref" / "libfdtdref.so"


def _reference_dir() -> Path:
    """Where the reference's sources are read from: $MPIFDTD_REFERENCE, else
    the REF default of the recipe that compiles them (oracle/ref.mk)."""
    env = os.environ.get("MPIFDTD_REFERENCE")
    if env:
        return Path(env)
    for line in (HERE / "ref.mk").read_text().splitlines():
        if line.startswith("REF") and "?=" in line:
            return Path(line.split("?=", 1)[1].strip())
    return HERE / "_ref" / "src"   # a directory that does not exist: reference absent


REF_SRC = _reference_dir()

# simulator.h:8-18
TM_UPML_2D, TE_UPML_2D, MPI_TM_UPML_2D, MPI_TE_UPML_2D = 2, 3, 4, 5
TM_2D, TE_2D, NS_TM_2D, NS_TE_2D = 0, 1, 6, 7
SOLVERS = {"TM_UPML": TM_UPML_2D, "TE_UPML": TE_UPML_2D,
           "MPI_TM_UPML": MPI_TM_UPML_2D, "MPI_TE_UPML": MPI_TE_UPML_2D,
           "TM_2D": TM_2D, "TE_2D": TE_2D, "NS_TM_2D": NS_TM_2D, "NS_TE_2D": NS_TE_2D}
MODEL_NONE, MODEL_CIRCLE, MODEL_MORPHO, MODEL_DISCS, MODEL_ZIGZAG = 0, 1, 2, 3, 4
NFFT = 8192


@dataclass
class FieldInfo:
    """field.h:20-28 FieldInfo (all physical sizes in nm), plus the settings the
    reference hard-codes (0 = its value): Courant number (0.7071, field.h:70),
    sigma grading exponent (2, field.c:259-283), NTFF inset in cells (5,
    field.c:136-139).  RefSim takes the reference's values only."""
    width_nm: int
    height_nm: int
    h_u_nm: int
    pml: int
    lambda_nm: int
    angle_deg: int
    step_num: int
    courant: float = 0.0
    pml_order: int = 0
    ntff_inset: int = 0

    def astuple(self):
        return (self.width_nm, self.height_nm, self.h_u_nm, self.pml,
                self.lambda_nm, self.angle_deg, self.step_num)


@dataclass
class Model:
    """kind + parameter vector, as ``of_model`` in fdtd_oracle.h."""
    kind: int = MODEL_NONE
    p: list = field(default_factory=list)

    @staticmethod
    def none():
        return Model(MODEL_NONE, [])

    @staticmethod
    def circle(radius_nm, eps=0.0):
        return Model(MODEL_CIRCLE, [float(radius_nm), float(eps)])

    @staticmethod
    def morpho(width_nm=300, thick0_nm=90, thick1_nm=90, layers=6, branch_nm=0,
               edge_rate=0.0, eps=0.0, widths_nm=None):
        p = [width_nm, thick0_nm, thick1_nm, layers, branch_nm, edge_rate, eps]
        if widths_nm is not None:
            p += [1.0] + [float(w) for w in widths_nm]
        else:
            p += [0.0]
        return Model(MODEL_MORPHO, [float(v) for v in p])

    @staticmethod
    def zigzag(width_nm=300, thickness_nm=80, layers=5, degree=10, n=0.0):
        """zigzagModel.c: lamellae at `degree` zig-zagging up; n <= 0: N_0 = 1.56."""
        return Model(MODEL_ZIGZAG, [float(width_nm), float(thickness_nm), float(layers), float(degree), float(n)])

    @staticmethod
    def discs(discs):
        """discs: iterable of (cx, cy, r, eps) in cell units (<= 8)."""
        discs = list(discs)[:8]
        p = [float(len(discs))]
        for d in discs:
            p += [float(v) for v in d]
        return Model(MODEL_DISCS, p)


class _OfFieldInfo(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("width_nm", "height_nm", "h_u_nm", "pml",
                                       "lambda_nm", "angle_deg", "step_num")] + \
               [("courant", C.c_double), ("pml_order", C.c_int), ("ntff_inset", C.c_int)]


class _OfModel(C.Structure):
    _fields_ = [("kind", C.c_int), ("p", C.c_double * 40)]


def _cc():
    return os.environ.get("CC", "gcc")


def build_oracle(force: bool = False) -> Path:
    """Compile fdtd_oracle.c into oracle/_build (portable flags, no -march)."""
    src = HERE / "fdtd_oracle.c"
    if force or not ORACLE_SO.exists() or ORACLE_SO.stat().st_mtime < src.stat().st_mtime:
        ORACLE_SO.parent.mkdir(parents=True, exist_ok=True)
        subprocess.run([_cc(), "-std=gnu99", "-O3", "-fPIC", "-ffp-contract=off", "-shared",
                        "-o", str(ORACLE_SO), str(src), "-lm", "-lpthread"], check=True)
    return ORACLE_SO


def reference_available() -> bool:
    return (REF_SRC / "mpiTM_UPML.c").exists()


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference sources with oracle/ref.mk when they are present."""
    if not reference_available():
        return REF_SO if REF_SO.exists() else None
    args = ["make", "-s", "-f", str(HERE / "ref.mk"), f"REF={REF_SRC}"]
    if force:
        args.insert(1, "-B")
    subprocess.run(args, check=True, cwd=str(HERE.parent))
    return REF_SO


_oracle_lib = None


def oracle_lib():
    global _oracle_lib
    if _oracle_lib is None:
        lib = C.CDLL(str(build_oracle()))
        P = C.c_void_p
        lib.of_create.restype = P
        lib.of_create.argtypes = [C.c_int, C.POINTER(_OfFieldInfo), C.POINTER(_OfModel)]
        lib.of_destroy.argtypes = [P]
        lib.of_step.argtypes = [P, C.c_int]
        lib.of_time.restype = C.c_double
        lib.of_time.argtypes = [P]
        lib.of_dims.argtypes = [P] + [C.POINTER(C.c_int)] * 4
        for fn in (lib.of_field, lib.of_eps, lib.of_ntff):
            fn.restype = C.POINTER(C.c_double)
            fn.argtypes = [P, C.c_int]
        lib.of_ntff_info.restype = C.c_int
        lib.of_ntff_info.argtypes = [P] + [C.POINTER(C.c_int)] * 6 + [C.POINTER(C.c_double)]
        lib.of_array_size.restype = C.c_int
        lib.of_array_size.argtypes = [P]
        lib.of_ntff_guard.restype = C.c_int
        lib.of_time_output.restype = C.c_int
        lib.of_time_output.argtypes = [P, C.POINTER(C.c_double)]
        lib.of_frequency.restype = C.c_int
        lib.of_frequency.argtypes = [P, C.POINTER(C.c_double)]
        lib.of_bench.restype = C.c_double
        lib.of_bench.argtypes = [C.c_int, C.POINTER(_OfFieldInfo), C.POINTER(_OfModel), C.c_int, C.c_int]
        lib.of_bench_opts.restype = C.c_double
        lib.of_bench_opts.argtypes = [C.c_int, C.POINTER(_OfFieldInfo), C.POINTER(_OfModel), C.c_int, C.c_int,
                                      C.c_int]
        _oracle_lib = lib
    return _oracle_lib


def _pack(fi: FieldInfo, m: Model):
    cfi = _OfFieldInfo(*fi.astuple(), float(fi.courant), int(fi.pml_order), int(fi.ntff_inset))
    cm = _OfModel()
    cm.kind = m.kind
    for i, v in enumerate(m.p[:40]):
        cm.p[i] = v
    return cfi, cm


def _cview(ptr, n):
    return np.ctypeslib.as_array(ptr, shape=(2 * n,)).view(np.complex128)


class OracleSim:
    """One simulation of the C restatement (fdtd_oracle.c)."""

    def __init__(self, solver, fi: FieldInfo, model: Model | None = None):
        self.lib = oracle_lib()
        self.solver = SOLVERS[solver] if isinstance(solver, str) else solver
        self.fi = fi
        self.model = model or Model.none()
        cfi, cm = _pack(fi, self.model)
        self.h = self.lib.of_create(self.solver, C.byref(cfi), C.byref(cm))
        if not self.h:
            raise ValueError("oracle rejected the configuration")
        d = [C.c_int() for _ in range(4)]
        self.lib.of_dims(self.h, *[C.byref(x) for x in d])
        self.nx, self.ny, self.n_px, self.n_py = (x.value for x in d)
        q = [C.c_int() for _ in range(6)]
        rf = C.c_double()
        self.array_size = self.lib.of_ntff_info(self.h, *[C.byref(x) for x in q], C.byref(rf))
        self.top, self.bottom, self.left, self.right, self.cx, self.cy = (x.value for x in q)
        self.rf = rf.value
        self.guard = self.lib.of_ntff_guard()

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.of_destroy(h)
            self.h = None

    @property
    def tm(self):
        return self.solver in (TM_UPML_2D, MPI_TM_UPML_2D)

    @property
    def mpi(self):
        return self.solver in (MPI_TM_UPML_2D, MPI_TE_UPML_2D)

    def step(self, n=1):
        self.lib.of_step(self.h, int(n))

    @property
    def time(self):
        return self.lib.of_time(self.h)

    def field(self, which):
        return _cview(self.lib.of_field(self.h, which), self.nx * self.ny).reshape(self.nx, self.ny).copy()

    def eps(self, which):
        p = self.lib.of_eps(self.h, which)
        return np.ctypeslib.as_array(p, shape=(self.nx * self.ny,)).reshape(self.nx, self.ny).copy()

    def ntff(self, which, with_guard=False):
        n = 360 * self.array_size + 2 * self.guard
        a = _cview(self.lib.of_ntff(self.h, which), n).copy()
        return a if with_guard else a[self.guard:self.guard + 360 * self.array_size]

    def time_output(self):
        out = np.zeros(321 * 360)
        rc = self.lib.of_time_output(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != 0:
            raise ValueError("spectrum needs step_num <= 8192")
        return out.reshape(321, 360)

    def frequency(self):
        out = np.zeros(720)
        rc = self.lib.of_frequency(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != 0:
            raise ValueError("frequency-domain NTFF failed")
        return out.view(np.complex128)


def oracle_bench(solver, fi: FieldInfo, model: Model, steps: int, threads: int, ntff: bool = True) -> float:
    """Wall seconds for `threads` independent simulations of `steps` steps
    (ntff=False: the MPI solvers leave out their time-domain NTFF)."""
    lib = oracle_lib()
    cfi, cm = _pack(fi, model)
    s = SOLVERS[solver] if isinstance(solver, str) else solver
    return lib.of_bench_opts(s, C.byref(cfi), C.byref(cm), int(steps), int(threads), 0 if ntff else 1)


_ref_lib = None


def ref_lib():
    global _ref_lib
    if _ref_lib is None:
        so = build_ref()
        if so is None or not Path(so).exists():
            raise FileNotFoundError("the reference oracle (oracle/_ref) is not built here")
        lib = C.CDLL(str(so))
        lib.refh_setup.restype = C.c_int
        lib.refh_setup.argtypes = [C.c_int] * 8 + [C.c_int, C.POINTER(C.c_double), C.c_void_p]
        lib.refh_step.argtypes = [C.c_int]
        lib.refh_discs_callback.restype = C.c_void_p
        lib.refh_discs_callback.argtypes = [C.c_int, C.POINTER(C.c_double)]
        for pre in ("mpitm", "mpite", "sertm", "serte"):
            for suf in ("field", "ntff"):
                f = getattr(lib, f"refh_{pre}_{suf}")
                f.restype = C.c_void_p
                f.argtypes = [C.c_int]
            f = getattr(lib, f"refh_{pre}_eps")
            f.restype = C.c_void_p
            f.argtypes = [C.c_int]
        for pre in ("splittm", "splitte", "nstm", "nste"):
            for suf in ("field", "eps"):
                f = getattr(lib, f"refh_{pre}_{suf}")
                f.restype = C.c_void_p
                f.argtypes = [C.c_int]
        for pre in ("mpitm", "mpite"):
            getattr(lib, f"refh_{pre}_dims").argtypes = [C.POINTER(C.c_int)] * 2
        lib.field_getTime.restype = C.c_double
        lib.refh_tm_frequency.argtypes = [C.c_void_p] * 4
        _ref_lib = lib
    return _ref_lib


class RefSim:
    """The reference itself (one at a time: it keeps global state)."""

    _PRE = {MPI_TM_UPML_2D: "mpitm", MPI_TE_UPML_2D: "mpite", TM_UPML_2D: "sertm", TE_UPML_2D: "serte",
            TM_2D: "splittm", TE_2D: "splitte", NS_TM_2D: "nstm", NS_TE_2D: "nste"}

    def __init__(self, solver, fi: FieldInfo, model: Model | None = None):
        if fi.courant or fi.pml_order or fi.ntff_inset:
            raise ValueError("the reference hard-codes the Courant number, sigma grading and NTFF inset")
        self.lib = ref_lib()
        self.solver = SOLVERS[solver] if isinstance(solver, str) else solver
        self.fi = fi
        model = model or Model.none()
        cb = None
        if model.kind == MODEL_DISCS:
            n = int(model.p[0])
            arr = (C.c_double * (4 * n))(*model.p[1:1 + 4 * n])
            cb = self.lib.refh_discs_callback(n, arr)
            mp = (C.c_double * 8)()
        else:
            vals = list(model.p) + [0.0] * 8
            mp = (C.c_double * 8)(*vals[:8])
        rc = self.lib.refh_setup(self.solver, *fi.astuple(), 3 if model.kind == MODEL_DISCS else model.kind, mp, cb)
        if rc != 0:
            raise ValueError(f"reference setup failed ({rc})")
        self.pre = self._PRE[self.solver]
        n_px = fi.width_nm // fi.h_u_nm
        n_py = fi.height_nm // fi.h_u_nm
        if self.solver in (MPI_TM_UPML_2D, MPI_TE_UPML_2D):
            a, b = C.c_int(), C.c_int()
            getattr(self.lib, f"refh_{self.pre}_dims")(C.byref(a), C.byref(b))
            self.nx, self.ny = a.value, b.value
        else:
            self.nx, self.ny = n_px, n_py
        self.n_px, self.n_py = n_px, n_py
        pml = fi.pml
        self.top, self.bottom = n_py - pml - 5, pml + 5
        self.left, self.right = pml + 5, n_px - pml - 5
        self.rf = 2.0 * ((self.top - self.bottom) // 2)
        self.array_size = int(fi.step_num + 2 * self.rf)

    def step(self, n=1):
        self.lib.refh_step(int(n))

    @property
    def time(self):
        return self.lib.field_getTime()

    def field(self, which):
        p = getattr(self.lib, f"refh_{self.pre}_field")(which)
        return _cview(C.cast(p, C.POINTER(C.c_double)), self.nx * self.ny).reshape(self.nx, self.ny).copy()

    def eps(self, which):
        p = getattr(self.lib, f"refh_{self.pre}_eps")(which)
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_double)), shape=(self.nx * self.ny,)).reshape(
            self.nx, self.ny).copy()

    def ntff(self, which):
        p = getattr(self.lib, f"refh_{self.pre}_ntff")(which)
        return _cview(C.cast(p, C.POINTER(C.c_double)), 360 * self.array_size).copy()

    def time_output(self, workdir):
        """Run the reference's ntff*_TimeOutput in `workdir`; return double[321][360]."""
        cwd = os.getcwd()
        os.makedirs(workdir, exist_ok=True)
        os.chdir(workdir)
        try:
            getattr(self.lib, f"refh_{self.pre}_time_output")()
        finally:
            os.chdir(cwd)
        f = Path(workdir) / f"{self.fi.angle_deg}[deg]_380nm_700nm_b.dat"
        return np.fromfile(f, dtype=np.float64).reshape(321, 360)

    def frequency_from(self, ez, hx, hy):
        """ntffTM_Frequency on global-frame (N_PX x N_PY) arrays."""
        ez, hx, hy = (np.ascontiguousarray(a, dtype=np.complex128) for a in (ez, hx, hy))
        res = np.zeros(360, dtype=np.complex128)
        self.lib.refh_tm_frequency(hx.ctypes.data, hy.ctypes.data, ez.ctypes.data, res.ctypes.data)
        return res


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    if den == 0:
        return float(num)
    return float(num / den)
