"""Batched engine (fdtd_batch_*): instances of uneven grids and step counts
advanced together must give what each gives alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _engine():
    import mpifdtd_gb300 as m
    return m


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# uneven grids, wavelengths and step counts (not multiples of the depth)
FIS = [(1200, 1200, 5, 10, 400, 0, 203), (1630, 1630, 5, 10, 500, 0, 158), (905, 905, 5, 10, 380, 0, 77),
       (2210, 2210, 5, 10, 640, 0, 251)]
MODELS = [(250.0, 2.25), (400.0, 3.1), (150.0, 1.6), (600.0, 2.43)]


def _single(m, solver, fi, model, precision="f64"):
    s = m.Simulation(solver, m.FieldInfo(*fi), precision)
    s.set_option(m.OPT_NTFF_MODE, 3)
    s.fill_model(m.MODEL_CIRCLE, list(model))
    s.run(fi[6])
    return s


@pytest.mark.parametrize("solver,k", [("MPI_TM_UPML", 4), ("MPI_TM_UPML", 1), ("MPI_TE_UPML", 2),
                                      ("MPI_TE_UPML", 4)])
def test_batch_fp64_equals_single_simulations(solver, k):
    m = _engine()
    b = m.Batch(solver, [m.FieldInfo(*fi) for fi in FIS], "f64")
    b.set_option(m.OPT_TBLOCK, k)
    for s, mdl in zip(b.instances, MODELS):
        s.fill_model(m.MODEL_CIRCLE, list(mdl))
    b.run()
    for i, (fi, mdl) in enumerate(zip(FIS, MODELS)):
        ref = _single(m, solver, fi, mdl)
        got = b.instances[i]
        assert got.time == fi[6]
        for w in range(3):
            e = _rel(got.field(w), ref.field(w))
            assert e <= TOL, (solver, k, i, w, e)
        if solver == "MPI_TM_UPML":
            assert _rel(got.frequency(), ref.frequency()) <= TOL
        ref.close()
    b.close()


def test_batch_rerun_after_reset_is_identical():
    m = _engine()
    b = m.Batch("MPI_TM_UPML", [m.FieldInfo(*fi) for fi in FIS[:3]], "f32")
    for s, mdl in zip(b.instances, MODELS):
        s.fill_model(m.MODEL_CIRCLE, list(mdl))
    b.run()
    first = [s.field(0) for s in b.instances]
    with pytest.raises(m.FdtdError):
        b.run()  # instances are at their step_num
    b.reset()
    b.run()
    for s, f in zip(b.instances, first):
        np.testing.assert_array_equal(s.field(0), f)
    b.close()


@pytest.mark.parametrize("k,cols", [(2, 1), (4, 1), (8, 1), (2, 2), (4, 2)])
def test_batch_fp32_farfield_within_1e3_of_fp64(k, cols):
    """FP32 fields (FP64 far-field sums) against the FP64 engine."""
    from mpifdtd_gb300.sweep import farfield_rel_err, mie_sweep, run_batch, run_sequential
    cases = mie_sweep(6)
    ff32, _, _, _ = run_batch(cases, "f32", tblock=k, cols=cols)
    ff64, _, _ = run_sequential(cases, "f64")
    err = farfield_rel_err(ff32, ff64)
    assert err.max() <= 1e-3, err
