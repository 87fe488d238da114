"""fdtd_ntff_step_noalloc: the NTFF step for callers that may not allocate.

Some callers own every device buffer themselves (a host application's memory
manager) or cannot afford the device-wide synchronisation of cudaMalloc in
their time loop.  They keep fields and NTFF accumulators in their own buffers
and call fdtd_ntff_step_noalloc once per update(); the library stages the
path samples in a static __device__ array instead of allocating.  This test
plays such a caller: it allocates its own accumulators (torch, outside the
library), reads the engine's device fields, and checks two calls in a row
against the engine's own NTFF accumulation (fdtd_run + fdtd_get_ntff) at the
1e-12 relative-L2 tolerance of the parity tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class _Config(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("width_nm", "height_nm", "h_u_nm", "pml", "lambda_nm",
                                       "angle_deg", "step_num", "precision", "flags", "courant_e4",
                                       "pml_order", "ntff_inset")] + [("reserved", C.c_int * 4)]


class _StepArgs(C.Structure):
    _fields_ = [("solver", C.c_int), ("cfg", _Config), ("e0", C.c_void_p), ("e1", C.c_void_p),
                ("h0", C.c_void_p), ("h1", C.c_void_p), ("pitch", C.c_int), ("time", C.c_double),
                ("acc", C.c_void_p * 3)]


GUARD = 16       # FDTD_NTFF_GUARD
MAX_PATH = 65536  # FDTD_NOALLOC_MAX_PATH


def _rel(a, b):
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / d) if d else float(np.linalg.norm(a - b))


def _device_field(lib, sim, which):
    p, pitch, rows = C.c_void_p(), C.c_int(), C.c_int()
    assert lib.fdtd_device_field(sim.h, which, C.byref(p), C.byref(pitch), C.byref(rows)) == 0
    return p.value, pitch.value


CANARY = 64      # complex elements past each guard that no call may touch
# an FP64 NaN payload no arithmetic produces: a write over it shows as a changed bit pattern
CANARY_BITS = np.uint64(0x7FF4DEADBEEFCAFE)

CASES = {
    # solver, FieldInfo (width, height, h_u, pml, lambda, angle, step_num), circle radius (nm), warm-up steps
    "tm_small": ("MPI_TM_UPML", (300, 320, 5, 6, 100, 0, 150), 60.0, 60),
    "te_small": ("MPI_TE_UPML", (300, 320, 5, 6, 100, 0, 150), 60.0, 60),
    # 100 x 32700 cells: a path of 65 480 cells, just under the 65 536 the static scratch holds
    "tm_path_near_cap": ("MPI_TM_UPML", (500, 163500, 5, 10, 100, 0, 200), 150.0, 30),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_noalloc_ntff_step_matches_engine(case):
    import torch

    import mpifdtd_gb300 as m

    solver, fi_t, radius, warm = CASES[case]
    lib = m.load()
    lib.fdtd_ntff_step_noalloc.restype = C.c_int
    lib.fdtd_ntff_step_noalloc.argtypes = [C.POINTER(_StepArgs), C.c_void_p]
    fi = m.FieldInfo(*fi_t)
    sim = m.Simulation(solver, fi)
    sim.fill_model(m.MODEL_CIRCLE, [radius, 0.0])
    sim.run(warm)
    before = [sim.ntff(w) for w in range(3)]
    before_guard = [sim.ntff_guard(w) for w in range(3)]

    n_block = 360 * sim.array_size
    # the caller's own accumulators: [canary | guard | block | guard | canary] per array
    n_all = n_block + 2 * GUARD + 2 * CANARY
    acc = torch.zeros((3, 2 * n_all), dtype=torch.float64, device="cuda")
    bits = acc.view(torch.int64)
    canary = int(CANARY_BITS.view(np.int64))
    bits[:, :2 * CANARY] = canary
    bits[:, 2 * (n_all - CANARY):] = canary
    tm = solver == "MPI_TM_UPML"
    fields = [_device_field(lib, sim, w) for w in range(3)]
    args = _StepArgs()
    args.solver = m.SOLVERS[solver]
    (args.cfg.width_nm, args.cfg.height_nm, args.cfg.h_u_nm, args.cfg.pml, args.cfg.lambda_nm,
     args.cfg.angle_deg, args.cfg.step_num) = fi.astuple()
    args.cfg.precision = m.F64
    if tm:   # Ez, Hx, Hy
        args.e0, args.e1, args.h0, args.h1 = fields[0][0], None, fields[1][0], fields[2][0]
    else:    # Ex, Ey, Hz
        args.e0, args.e1, args.h0, args.h1 = fields[0][0], fields[1][0], fields[2][0], None
    args.pitch = fields[0][1]
    for w in range(3):
        args.acc[w] = acc[w].data_ptr() + (CANARY + GUARD) * 16
    torch.cuda.synchronize()

    for call in range(2):                     # two calls in a row
        t = sim.time
        sim.run(1)                            # the engine's own update() of this step
        sim.synchronize()
        args.time = t
        rc = lib.fdtd_ntff_step_noalloc(C.byref(args), C.c_void_p(sim.stream))
        assert rc == 0, lib.fdtd_last_error().decode()
        sim.synchronize()
        torch.cuda.synchronize()
        host = acc.cpu().numpy()
        got = host.view(np.complex128)
        wants = [sim.ntff(w) - before[w] for w in range(3)]   # the engine's accumulation of the same steps
        # (on the tall grid the far top and bottom sides see no field yet: their accumulator stays zero)
        assert max(np.abs(x).max() for x in wants) > 0
        for w in range(3):
            want = wants[w]
            err = _rel(got[w, CANARY + GUARD:CANARY + GUARD + n_block], want)
            assert err <= 1e-12, (case, call, w, err)
            # guard cells: what the engine's flat index spilled there over the same steps
            g_want = sim.ntff_guard(w) - before_guard[w]
            g_got = np.concatenate([got[w, CANARY:CANARY + GUARD],
                                    got[w, CANARY + GUARD + n_block:CANARY + 2 * GUARD + n_block]])
            assert np.abs(g_got - g_want).max() <= 1e-12 * max(1.0, np.abs(want).max()), (case, call, w)
            # nothing beyond the guards is written
            raw = host[w].view(np.uint64)
            assert np.all(raw[:2 * CANARY] == CANARY_BITS), (case, call, w, "front canary")
            assert np.all(raw[2 * (n_all - CANARY):] == CANARY_BITS), (case, call, w, "back canary")
    assert sim.status == 0


def test_noalloc_rejects_path_beyond_static_scratch():
    import mpifdtd_gb300 as m

    lib = m.load()
    lib.fdtd_ntff_step_noalloc.restype = C.c_int
    lib.fdtd_ntff_step_noalloc.argtypes = [C.POINTER(_StepArgs), C.c_void_p]
    args = _StepArgs()
    args.solver = m.MPI_TM_UPML_2D
    side = (MAX_PATH // 4 + 200) * 2          # a path longer than the scratch holds
    (args.cfg.width_nm, args.cfg.height_nm, args.cfg.h_u_nm, args.cfg.pml, args.cfg.lambda_nm,
     args.cfg.angle_deg, args.cfg.step_num) = (side, side, 2, 16, 500, 0, 100)
    args.e0 = args.h0 = args.h1 = 1           # never dereferenced: rejected before any launch
    args.pitch = side
    args.acc[0] = args.acc[1] = args.acc[2] = 1
    assert lib.fdtd_ntff_step_noalloc(C.byref(args), None) == 1   # FDTD_E_ARG
    assert b"static scratch" in lib.fdtd_last_error()
