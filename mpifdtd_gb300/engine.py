"""Python binding of the C ABI in include/mpifdtd_gb300.h (ctypes).

The native library is required: importing this module on a machine where the
library was not built raises, and creating a Simulation without a CUDA device
fails with the engine's own error.  There is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import build as _build

# simulator.h:8-18 enum SOLVER values
TM_2D, TE_2D, TM_UPML_2D, TE_UPML_2D, MPI_TM_UPML_2D, MPI_TE_UPML_2D, NS_TM_2D, NS_TE_2D = range(8)
SOLVERS = {"TM_UPML": TM_UPML_2D, "TE_UPML": TE_UPML_2D,
           "MPI_TM_UPML": MPI_TM_UPML_2D, "MPI_TE_UPML": MPI_TE_UPML_2D,
           "TM_2D": TM_2D, "TE_2D": TE_2D, "NS_TM_2D": NS_TM_2D, "NS_TE_2D": NS_TE_2D}
F64, F32 = 0, 1
LAYOUT_GLOBAL, LAYOUT_SOLVER = 0, 1
MODEL_NONE, MODEL_CIRCLE, MODEL_MORPHO, MODEL_ZIGZAG = 0, 1, 3, 5
OPT_NTFF_MODE, OPT_NTFF_CHUNK, OPT_NTFF_BLOCK, OPT_ROWS = 1, 2, 3, 4
OPT_TBLOCK, OPT_TBLOCK_ROWS, OPT_TBLOCK_COLS, OPT_DFT_STRIDE = 5, 6, 7, 8

_ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "bad state", 5: "unsupported"}


class FdtdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_ERRORS.get(code, code)}: {msg}")
        self.code = code


@dataclass
class FieldInfo:
    """field.h:20-28 FieldInfo (physical sizes in nm), plus three settings the
    reference hard-codes (0 keeps the reference's value): the Courant number
    (C_0_S = 0.7071, field.h:70; given to the engine in units of 1e-4), the
    sigma grading exponent (2, field.c:259-283) and the NTFF path's distance
    from the PML in cells (5, field.c:136-139)."""
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
        return (self.width_nm, self.height_nm, self.h_u_nm, self.pml, self.lambda_nm,
                self.angle_deg, self.step_num)


class _Config(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("width_nm", "height_nm", "h_u_nm", "pml", "lambda_nm",
                                       "angle_deg", "step_num", "precision", "flags", "courant_e4",
                                       "pml_order", "ntff_inset")] + [("reserved", C.c_int * 4)]


class Geometry(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("n_px", "n_py", "n_pml", "n_x", "n_y", "ntff_top", "ntff_bottom",
                                       "ntff_left", "ntff_right", "ntff_cx", "ntff_cy")] + \
               [("rf_per_c", C.c_double), ("array_size", C.c_int), ("lambda_s", C.c_double),
                ("k_s", C.c_double), ("omega_s", C.c_double)]


_lib = None


def library_path() -> Path:
    return _build.ENGINE_SO


def load():
    """Load the engine library (built by mpifdtd_gb300.build / __graft_entry__.build)."""
    global _lib
    if _lib is not None:
        return _lib
    so = library_path()
    if not so.exists():
        raise ImportError(f"mpifdtd_gb300 engine library missing ({so}); run mpifdtd_gb300.build.build()")
    lib = C.CDLL(str(so))
    P, I, D = C.c_void_p, C.c_int, C.c_double
    dp = C.POINTER(C.c_double)
    sig = {
        "fdtd_geometry_of": (I, [C.POINTER(_Config), C.POINTER(Geometry)]),
        "fdtd_create": (I, [I, C.POINTER(_Config), C.POINTER(P)]),
        "fdtd_destroy": (I, [P]),
        "fdtd_get_geometry": (I, [P, C.POINTER(Geometry)]),
        "fdtd_set_eps": (I, [P, dp, dp, dp]),
        "fdtd_fill_eps_model": (I, [P, I, dp, I]),
        "fdtd_update": (I, [P, D, D]),
        "fdtd_run": (I, [P, I]),
        "fdtd_get_time": (I, [P, dp]),
        "fdtd_set_time": (I, [P, D]),
        "fdtd_synchronize": (I, [P]),
        "fdtd_flush": (I, [P]),
        "fdtd_get_field": (I, [P, I, I, dp]),
        "fdtd_get_eps": (I, [P, I, I, dp]),
        "fdtd_get_ntff": (I, [P, I, dp]),
        "fdtd_get_ntff_guard": (I, [P, I, dp, C.POINTER(I)]),
        "fdtd_reset": (I, [P]),
        "fdtd_device_field": (I, [P, I, C.POINTER(P), C.POINTER(I), C.POINTER(I)]),
        "fdtd_launch_count": (C.c_longlong, [P]),
        "fdtd_get_status": (I, [P, C.POINTER(C.c_uint)]),
        "fdtd_get_stream": (I, [P, C.POINTER(P)]),
        "fdtd_spectrum": (I, [P, dp]),
        "fdtd_frequency": (I, [P, dp]),
        "fdtd_elliptic": (I, [P, I, dp]),
        "fdtd_write_elliptic": (I, [P, I, C.c_char_p]),
        "fdtd_write_model_image": (I, [P, I, C.c_char_p]),
        "fdtd_profile_enable": (I, [P, I]),
        "fdtd_profile_read": (I, [P, dp, C.POINTER(C.c_longlong)]),
        "fdtd_set_option": (I, [P, I, I]),
        "fdtd_get_option": (I, [P, I, C.POINTER(I)]),
        "fdtd_autotune": (I, [P, C.POINTER(I), C.POINTER(I), dp]),
        "fdtd_autotune_report": (I, [P, dp, I]),
        "fdtd_dft_enable": (I, [P, I, C.POINTER(I)]),
        "fdtd_dft_far_field": (I, [P, dp]),
        "fdtd_dft_spectrum": (I, [P, dp]),
        "fdtd_batch_create": (I, [I, P, I, C.POINTER(P)]),
        "fdtd_batch_destroy": (I, [P]),
        "fdtd_batch_size": (I, [P]),
        "fdtd_batch_instance": (I, [P, I, C.POINTER(P)]),
        "fdtd_batch_set_option": (I, [P, I, I]),
        "fdtd_batch_run": (I, [P]),
        "fdtd_batch_reset": (I, [P]),
        "fdtd_batch_launch_count": (C.c_longlong, [P]),
        "fdtd_batch_broadband": (I, [P, I, C.POINTER(I)]),
        "fdtd_batch_broadband_spectrum": (I, [P, I, dp]),
        "fdtd_batch_broadband_spectra": (I, [P, dp]),
        "fdtd_check_finite": (I, [P, C.POINTER(C.c_longlong)]),
        "fdtd_checkpoint_size": (I, [P, C.POINTER(C.c_size_t)]),
        "fdtd_checkpoint_save": (I, [P, P, C.c_size_t]),
        "fdtd_checkpoint_load": (I, [P, P, C.c_size_t]),
        "fdtd_checkpoint_write": (I, [P, C.c_char_p]),
        "fdtd_checkpoint_read": (I, [P, C.c_char_p]),
        "fdtd_last_error": (C.c_char_p, []),
        "fdtd_version": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _check(rc):
    if rc != 0:
        raise FdtdError(rc, load().fdtd_last_error().decode())


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


CFG_NO_TIME_NTFF = 1
STATUS_NTFF_RANGE = 1
STATUS_NONFINITE = 4


def _config(fi: FieldInfo, precision: int, flags: int = 0) -> _Config:
    c = _Config()
    (c.width_nm, c.height_nm, c.h_u_nm, c.pml, c.lambda_nm, c.angle_deg, c.step_num) = fi.astuple()
    c.precision = precision
    c.flags = flags
    e4 = round(fi.courant * 1e4)
    if abs(fi.courant * 1e4 - e4) > 1e-6:
        raise ValueError(f"Courant number {fi.courant} is not a multiple of 1e-4")
    c.courant_e4, c.pml_order, c.ntff_inset = e4, fi.pml_order, fi.ntff_inset
    return c


def geometry_of(fi: FieldInfo) -> Geometry:
    g = Geometry()
    _check(load().fdtd_geometry_of(C.byref(_config(fi, F64)), C.byref(g)))
    return g


class Simulation:
    """One GPU simulation of a UPML solver (see include/mpifdtd_gb300.h)."""

    def __init__(self, solver, fi: FieldInfo, precision: int | str = F64, _borrow=None, no_time_ntff=False):
        self.lib = load()
        self.solver = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        if isinstance(precision, str):
            precision = {"f64": F64, "f32": F32}[precision]
        self.precision = precision
        self.fi = fi
        h = C.c_void_p()
        if _borrow is not None:  # an instance owned by a Batch
            h, self._owner = _borrow
        else:
            flags = CFG_NO_TIME_NTFF if no_time_ntff else 0
            _check(self.lib.fdtd_create(self.solver, C.byref(_config(fi, precision, flags)), C.byref(h)))
        self.h = h
        self.geo = Geometry()
        _check(self.lib.fdtd_get_geometry(self.h, C.byref(self.geo)))

    # -- lifetime
    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owner", None) is None:
                self.lib.fdtd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- properties
    @property
    def tm(self):
        return self.solver in (TM_UPML_2D, MPI_TM_UPML_2D, TM_2D, NS_TM_2D)

    @property
    def mpi(self):
        return self.solver in (MPI_TM_UPML_2D, MPI_TE_UPML_2D)

    @property
    def n_px(self):
        return self.geo.n_px

    @property
    def n_py(self):
        return self.geo.n_py

    @property
    def array_size(self):
        return self.geo.array_size

    @property
    def time(self) -> float:
        t = C.c_double()
        _check(self.lib.fdtd_get_time(self.h, C.byref(t)))
        return t.value

    @time.setter
    def time(self, t):
        _check(self.lib.fdtd_set_time(self.h, float(t)))

    @property
    def status(self) -> int:
        f = C.c_uint()
        _check(self.lib.fdtd_get_status(self.h, C.byref(f)))
        return f.value

    @property
    def launches(self) -> int:
        return int(self.lib.fdtd_launch_count(self.h))

    # -- inputs
    def set_eps(self, e0, e1=None, e2=None):
        arrs = []
        for e in (e0, e1, e2):
            if e is None:
                arrs.append(None)
            else:
                e = np.ascontiguousarray(e, dtype=np.float64)
                if e.shape != (self.n_px, self.n_py):
                    raise ValueError(f"eps must be ({self.n_px}, {self.n_py}), got {e.shape}")
                arrs.append(e)
        _check(self.lib.fdtd_set_eps(self.h, *[_dptr(a) for a in arrs]))

    @property
    def stream(self) -> int:
        """cudaStream_t of this simulation (every launch goes there)."""
        p = C.c_void_p()
        _check(self.lib.fdtd_get_stream(self.h, C.byref(p)))
        return int(p.value or 0)

    def set_eps_ptr(self, e0: int, e1: int = 0, e2: int = 0):
        """Like set_eps, from raw host addresses (e.g. pinned buffers)."""
        dp = C.POINTER(C.c_double)
        _check(self.lib.fdtd_set_eps(self.h, *[C.cast(C.c_void_p(a), dp) if a else None for a in (e0, e1, e2)]))

    def field_into(self, which: int, host_addr: int, layout: int = LAYOUT_GLOBAL):
        """Copy a field to a raw host address (complex interleaved)."""
        _check(self.lib.fdtd_get_field(self.h, int(which), int(layout),
                                       C.cast(C.c_void_p(host_addr), C.POINTER(C.c_double))))

    def ntff_into(self, which: int, host_addr: int):
        _check(self.lib.fdtd_get_ntff(self.h, int(which), C.cast(C.c_void_p(host_addr), C.POINTER(C.c_double))))

    def eps_into(self, which: int, host_addr: int, layout: int = LAYOUT_GLOBAL):
        _check(self.lib.fdtd_get_eps(self.h, int(which), int(layout),
                                     C.cast(C.c_void_p(host_addr), C.POINTER(C.c_double))))

    def spectrum(self) -> np.ndarray:
        """|E|^2 far-field spectrum, double[321][360] (380..700 nm x angle)."""
        out = np.empty((321, 360), dtype=np.float64)
        _check(self.lib.fdtd_spectrum(self.h, _dptr(out)))
        return out

    def frequency(self) -> np.ndarray:
        """Frequency-domain NTFF of the current fields (360 complex): E_z far field
        (TM, ntffTM_Frequency) or E_phi (TE, ntffTE_Frequency)."""
        out = np.empty(360, dtype=np.complex128)
        _check(self.lib.fdtd_frequency(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def _e_index(self, which):
        """The E field the reference's outputs use: Ez (TM), Ey (TE)."""
        return (0 if self.tm else 1) if which is None else int(which)

    def elliptic(self, which=None) -> np.ndarray:
        """field_outputElliptic's ring: |E|^2 at 181 points of the 1.2 lambda
        circle, index q = 180 - angle (TM: Ez, TE: Ey unless `which`)."""
        out = np.empty(181)
        _check(self.lib.fdtd_elliptic(self.h, self._e_index(which), out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def write_elliptic(self, path, which=None):
        """The ring as field_outputElliptic's text file."""
        _check(self.lib.fdtd_write_elliptic(self.h, self._e_index(which), str(path).encode()))

    def write_model_image(self, path, which=None):
        """drawer_outputImage's 24-bit BMP of the permittivity the solver's
        getEps() returns (TM: EPS_EZ, TE: EPS_EY unless `which`), global frame."""
        _check(self.lib.fdtd_write_model_image(self.h, self._e_index(which), str(path).encode()))

    def profile(self, on: bool = True):
        """Record CUDA events around every launch class on the engine stream."""
        _check(self.lib.fdtd_profile_enable(self.h, 1 if on else 0))

    def profile_read(self) -> dict:
        """Summed ms per launch class since profile(True) (synchronizes, clears)."""
        ms = np.zeros(4)
        steps = C.c_longlong()
        _check(self.lib.fdtd_profile_read(self.h, _dptr(ms), C.byref(steps)))
        return {"e_half": ms[0], "h_half": ms[1], "ntff_gather": ms[2], "ntff_deposit": ms[3],
                "steps": int(steps.value)}

    def set_option(self, key: int, value: int):
        _check(self.lib.fdtd_set_option(self.h, int(key), int(value)))

    def get_option(self, key: int) -> int:
        v = C.c_int()
        _check(self.lib.fdtd_get_option(self.h, int(key), C.byref(v)))
        return v.value

    def dft_enable(self, lambdas_nm):
        """Running-DFT NTFF at these wavelengths (nm); call before the first step."""
        lam = np.ascontiguousarray(lambdas_nm, dtype=np.int32)
        self._dft_n = int(lam.size)
        _check(self.lib.fdtd_dft_enable(self.h, self._dft_n, lam.ctypes.data_as(C.POINTER(C.c_int))))

    def dft_far_field(self) -> np.ndarray:
        out = np.empty((360, 2 * self._dft_n), dtype=np.complex128)
        _check(self.lib.fdtd_dft_far_field(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def dft_spectrum(self) -> np.ndarray:
        """|E|^2 [n_lambda, 360] from the running DFT (the spectrum's interpolation)."""
        out = np.empty((self._dft_n, 360))
        _check(self.lib.fdtd_dft_spectrum(self.h, _dptr(out)))
        return out

    def autotune(self) -> dict:
        """Pick the temporal-blocking depth and tile rows on this grid (the
        fields do not change); returns them with the stencil ms per step."""
        k, rows, ms = C.c_int(), C.c_int(), C.c_double()
        _check(self.lib.fdtd_autotune(self.h, C.byref(k), C.byref(rows), C.byref(ms)))
        n = self.lib.fdtd_autotune_report(self.h, None, 0)
        table = np.zeros(4 * max(n, 0))
        self.lib.fdtd_autotune_report(self.h, _dptr(table), n)
        return {"tblock": k.value, "tblock_rows": rows.value, "tblock_cols": self.get_option(OPT_TBLOCK_COLS),
                "stencil_ms_per_step": ms.value,
                "candidates": [(int(a), int(b), int(c), float(d)) for a, b, c, d in table.reshape(-1, 4)]}

    def fill_model(self, model: int, params=()):
        p = np.ascontiguousarray(params, dtype=np.float64)
        _check(self.lib.fdtd_fill_eps_model(self.h, int(model), _dptr(p) if p.size else None, int(p.size)))

    # -- stepping
    def update(self, time: float, ray_coef: float):
        _check(self.lib.fdtd_update(self.h, float(time), float(ray_coef)))

    def run(self, n: int):
        _check(self.lib.fdtd_run(self.h, int(n)))

    def synchronize(self):
        _check(self.lib.fdtd_synchronize(self.h))

    def flush(self):
        """Enqueue the deposit of the buffered NTFF steps (fdtd_flush); no wait."""
        _check(self.lib.fdtd_flush(self.h))

    def reset(self):
        _check(self.lib.fdtd_reset(self.h))

    # -- failure detection, checkpoint / resume
    def check_finite(self) -> int:
        """Number of field values with a non-finite part (fdtd_check_finite);
        a non-zero count also sets STATUS_NONFINITE in `status`."""
        n = C.c_longlong()
        _check(self.lib.fdtd_check_finite(self.h, C.byref(n)))
        return n.value

    def checkpoint(self, path=None):
        """The simulation's state as a checkpoint image: written to `path`, or
        returned as a uint8 array when no path is given."""
        if path is not None:
            _check(self.lib.fdtd_checkpoint_write(self.h, os.fsencode(path)))
            return None
        n = C.c_size_t()
        _check(self.lib.fdtd_checkpoint_size(self.h, C.byref(n)))
        buf = np.empty(n.value, dtype=np.uint8)
        _check(self.lib.fdtd_checkpoint_save(self.h, buf.ctypes.data, n.value))
        return buf

    def restore(self, image):
        """Load a checkpoint image (a path, or the array `checkpoint()` returned)
        into this simulation, created with the same solver and FieldInfo."""
        if isinstance(image, (str, os.PathLike)):
            with open(image, "rb") as f:
                head = np.frombuffer(f.read(40), dtype=np.uint8)
            _check(self.lib.fdtd_checkpoint_read(self.h, os.fsencode(image)))
        else:
            buf = np.ascontiguousarray(image, dtype=np.uint8)
            head = buf[:40]
            _check(self.lib.fdtd_checkpoint_load(self.h, buf.ctypes.data, buf.size))
        nlam = int(head[36:40].view(np.int32)[0])     # the image's running-DFT wavelengths
        if nlam > 0:
            self._dft_n = nlam

    # -- outputs
    def _shape(self, layout):
        if layout == LAYOUT_SOLVER and self.mpi:
            return (self.n_px + 2, self.n_py + 2)
        return (self.n_px, self.n_py)

    def field(self, which: int, layout: int = LAYOUT_GLOBAL) -> np.ndarray:
        shp = self._shape(layout)
        out = np.empty(shp, dtype=np.complex128)
        _check(self.lib.fdtd_get_field(self.h, int(which), int(layout),
                                       out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def eps(self, which: int, layout: int = LAYOUT_GLOBAL) -> np.ndarray:
        out = np.empty(self._shape(layout), dtype=np.float64)
        _check(self.lib.fdtd_get_eps(self.h, int(which), int(layout), _dptr(out)))
        return out

    def ntff(self, which: int) -> np.ndarray:
        out = np.empty(360 * self.array_size, dtype=np.complex128)
        _check(self.lib.fdtd_get_ntff(self.h, int(which), out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def ntff_guard(self, which: int) -> np.ndarray:
        g = C.c_int()
        out = np.empty(64, dtype=np.complex128)
        _check(self.lib.fdtd_get_ntff_guard(self.h, int(which), out.ctypes.data_as(C.POINTER(C.c_double)),
                                            C.byref(g)))
        return out[:2 * g.value]


class Batch:
    """Independent instances of one MPI solver advanced together (fdtd_batch_*):
    a sweep of structures / wavelengths with uneven grids and step counts.

    batch.instances[i] is a Simulation view of instance i (owned by the batch):
    fill its permittivity before run(), read fields and frequency() after."""

    def __init__(self, solver, fis, precision: int | str = F32, no_time_ntff=True):
        self.lib = load()
        self.solver = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        if isinstance(precision, str):
            precision = {"f64": F64, "f32": F32}[precision]
        flags = CFG_NO_TIME_NTFF if no_time_ntff else 0
        cfgs = (_Config * len(fis))(*[_config(fi, precision, flags) for fi in fis])
        h = C.c_void_p()
        _check(self.lib.fdtd_batch_create(self.solver, cfgs, len(fis), C.byref(h)))
        self.h = h
        self.instances = []
        for i, fi in enumerate(fis):
            sh = C.c_void_p()
            _check(self.lib.fdtd_batch_instance(self.h, i, C.byref(sh)))
            self.instances.append(Simulation(self.solver, fi, precision, _borrow=(sh, self)))

    def set_option(self, key: int, value: int):
        _check(self.lib.fdtd_batch_set_option(self.h, int(key), int(value)))

    def run(self):
        """Every instance from time 0 to its own step_num."""
        _check(self.lib.fdtd_batch_run(self.h))

    def broadband(self, lambdas_nm):
        """Gaussian-pulse source and a running DFT of the NTFF path at these
        wavelengths (fdtd_batch_broadband); call before run()."""
        lam = np.ascontiguousarray(lambdas_nm, dtype=np.int32)
        self._bb_n = int(lam.size)
        _check(self.lib.fdtd_batch_broadband(self.h, self._bb_n, lam.ctypes.data_as(C.POINTER(C.c_int))))

    def broadband_spectrum(self, index: int) -> np.ndarray:
        """Far-field intensity [n_lambda, 360] of instance `index` per unit
        incident wave (fdtd_batch_broadband_spectrum); angle a is direction a."""
        out = np.empty((self._bb_n, 360))
        _check(self.lib.fdtd_batch_broadband_spectrum(self.h, int(index), _dptr(out)))
        return out

    def broadband_spectra(self) -> np.ndarray:
        """Far-field intensity [n, n_lambda, 360] of every instance (fdtd_batch_broadband_spectra)."""
        out = np.empty((len(self.instances), self._bb_n, 360))
        _check(self.lib.fdtd_batch_broadband_spectra(self.h, _dptr(out)))
        return out

    def reset(self):
        _check(self.lib.fdtd_batch_reset(self.h))

    @property
    def launches(self) -> int:
        return int(self.lib.fdtd_batch_launch_count(self.h))

    def close(self):
        if getattr(self, "h", None):
            for s in self.instances:
                s.h = None
            self.lib.fdtd_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
