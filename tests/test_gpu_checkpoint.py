"""Checkpoint / resume (fdtd_checkpoint_*) and the finite-value check
(fdtd_check_finite), through the C ABI.

A run interrupted by a checkpoint and resumed in a fresh simulation must end
where the uninterrupted run ends, with the buffered NTFF steps of the cut (37
steps: not a multiple of the 32-step deposit block) and the tuning options
carried over: fields and running-DFT far fields bit for bit, the time-domain
NTFF accumulators to rounding (their deposit adds with FP64 atomics in no
fixed order, so two runs of one simulation differ there at the 1e-16 level).
Failure detection is tested by injecting a NaN on the host: into a
checkpoint image, which is then loaded.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAMS = [400, 500, 600]
HEADER = 200  # bytes of the fixed checkpoint header (then 4 per DFT wavelength)


def _sim(solver, fi, precision="f64", tblock=0, dft=False, model=True):
    import mpifdtd_gb300 as m
    sim = m.Simulation(solver, m.FieldInfo(*fi), precision)
    if model:
        sim.fill_model(m.MODEL_CIRCLE, [120.0, 2.25])
    if tblock:
        sim.set_option(m.OPT_TBLOCK, tblock)
    if dft:
        sim.dft_enable(LAMS)
    return sim


def _state(sim):
    import mpifdtd_gb300 as m
    upml = sim.solver in (m.TM_UPML_2D, m.TE_UPML_2D, m.MPI_TM_UPML_2D, m.MPI_TE_UPML_2D)
    ntff = [sim.ntff(w) for w in range(3)] if upml else []   # NS / split-field: no time-domain NTFF
    return [sim.field(w) for w in range(3)], ntff


def _equal(a, b):
    for x, y in zip(a[0], b[0]):
        assert np.array_equal(x, y), np.abs(x - y).max()
    for x, y in zip(a[1], b[1]):
        assert np.abs(x - y).max() <= 1e-13 * np.abs(y).max(), np.abs(x - y).max() / np.abs(y).max()


CASES = [("MPI_TM_UPML", (400, 400, 5, 8, 500, 0, 200), "f64", 0, True),
         ("MPI_TM_UPML", (400, 400, 5, 8, 500, 0, 200), "f32", 4, True),
         ("MPI_TE_UPML", (400, 400, 5, 8, 500, 30, 200), "f64", 2, False),
         ("TM_UPML", (400, 400, 5, 8, 500, 0, 200), "f64", 0, True),
         ("TE_UPML", (400, 400, 5, 8, 500, 30, 200), "f64", 0, False),
         ("NS_TM_2D", (400, 400, 5, 8, 500, 0, 200), "f64", 0, False)]


@pytest.mark.parametrize("solver,fi,prec,tblock,dft", CASES)
@pytest.mark.parametrize("route", ["buffer", "file"])
def test_resumed_run_is_bit_identical(solver, fi, prec, tblock, dft, route, tmp_path):
    ref = _sim(solver, fi, prec, tblock, dft)
    ref.run(37)
    image = ref.checkpoint() if route == "buffer" else None
    if route == "file":
        ref.checkpoint(tmp_path / "sim.ckpt")
    ref.run(53)
    want = _state(ref)
    want_dft = ref.dft_far_field() if dft else None
    # a fresh simulation of the same configuration: no model, default options,
    # no running DFT -- all of it comes from the image
    res = _sim(solver, fi, prec, model=False)
    res.restore(image if route == "buffer" else tmp_path / "sim.ckpt")
    assert res.time == 37
    import mpifdtd_gb300 as m
    assert res.get_option(m.OPT_TBLOCK) == tblock
    assert np.array_equal(res.eps(0), ref.eps(0))
    res.run(53)
    assert res.time == ref.time == 90
    _equal(_state(res), want)
    if dft:
        assert np.array_equal(res.dft_far_field(), want_dft)
    ref.close()
    res.close()


def test_checkpoint_rejects_other_configurations_and_corrupt_images():
    import mpifdtd_gb300 as m
    fi = (400, 400, 5, 8, 500, 0, 200)
    a = _sim("MPI_TM_UPML", fi)
    a.run(10)
    img = a.checkpoint()
    for solver, other in [("MPI_TM_UPML", (400, 400, 5, 8, 520, 0, 200)),   # other wavelength
                          ("MPI_TE_UPML", fi),                                # other solver
                          ("MPI_TM_UPML", (420, 400, 5, 8, 500, 0, 200))]:    # other grid
        b = m.Simulation(solver, m.FieldInfo(*other))
        with pytest.raises(m.FdtdError):
            b.restore(img)
        b.close()
    b = m.Simulation("MPI_TM_UPML", m.FieldInfo(*fi), "f32")   # other precision
    with pytest.raises(m.FdtdError):
        b.restore(img)
    b.close()
    b = m.Simulation("MPI_TM_UPML", m.FieldInfo(*fi))
    with pytest.raises(m.FdtdError):
        b.restore(img[:-8])                                      # truncated
    bad = img.copy()
    bad[0] ^= 0xFF                                               # not an image
    with pytest.raises(m.FdtdError):
        b.restore(bad)
    b.dft_enable([450])
    c = _sim("MPI_TM_UPML", fi, dft=True)
    with pytest.raises(m.FdtdError):                             # other DFT wavelengths
        b.restore(c.checkpoint())
    c.close()
    # a rejected image leaves the simulation usable
    b.run(5)
    assert b.time == 5
    b.close()
    a.close()


def test_finite_check_finds_an_injected_nan_and_leaves_the_simulation_usable():
    import mpifdtd_gb300 as m
    fi = (400, 400, 5, 8, 500, 0, 200)
    sim = _sim("MPI_TM_UPML", fi)
    sim.run(20)
    assert sim.check_finite() == 0
    assert sim.status & m.STATUS_NONFINITE == 0
    img = sim.checkpoint()
    nxa, pitch = (int(v) for v in np.frombuffer(img[28:36].tobytes(), dtype=np.int32))
    cells = nxa * pitch
    # eps arrays, then the field slots (complex FP64): slot 1 is Dz, which the
    # E half-step accumulates (Ez = Dz / eps is recomputed from it every step)
    slot1 = HEADER + 3 * cells * 8 + cells * 16
    k = (nxa // 2) * pitch + pitch // 2            # a cell in the middle of the grid
    vals = img[slot1:slot1 + cells * 16].view(np.float64)
    vals[2 * k] = np.nan
    sim.restore(img)
    assert sim.check_finite() == 1
    assert sim.status & m.STATUS_NONFINITE
    sim.run(3)                                     # the NaN spreads; nothing traps
    assert sim.check_finite() > 1
    assert sim.time == 23
    sim.close()
