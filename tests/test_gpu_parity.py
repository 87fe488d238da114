"""GPU parity: the CUDA engine against the reference's golden vectors and the oracle.

Bar: FP64 fields and NTFF accumulators within 1e-12 relative L2
of the reference.  Permittivity is an input here: the golden ("full") cases
carry the reference's own eps arrays, the others take the oracle's.
"""
import numpy as np
import pytest

from tests.golden.cases import CASES, make_model
from tests.golden.golden_io import capture, compare, crop, rel

pytestmark = pytest.mark.gpu

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"
TOL = 1e-12


def _engine():
    import mpifdtd_gb300 as m
    return m


def _eps_for(name, c):
    ref = np.load(GOLDEN / f"{name}.npz")
    if "eps0" in ref:
        return [ref[f"eps{w}"] for w in range(3)]
    from oracle.pyoracle import FieldInfo as OFI, OracleSim
    o = OracleSim(c["solver"], OFI(*c["fi"]), make_model(c["model"]))
    mpi = c["solver"].startswith("MPI")
    return [crop(o.eps(w), mpi) for w in range(3)]


def run_gpu(name, precision="f64"):
    m = _engine()
    c = CASES[name]
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]), precision)
    sim.set_eps(*_eps_for(name, c))
    sim.run(c["steps"])
    fields = [sim.field(w) for w in range(3)]
    eps = [sim.eps(w) for w in range(3)]
    ntff = [] if c.get("no_ntff") else [sim.ntff(w) for w in range(3)]   # split-field / NS: no NTFF
    out = capture(fields, eps, ntff, sim.array_size, c["kind"], c.get("rows", "all"))
    extras = c.get("extras", ())
    if "spectrum" in extras:
        out["spectrum"] = sim.spectrum()
    if "frequency" in extras:
        out["frequency"] = sim.frequency()
    out["meta_time"] = np.array(sim.time)
    return sim, out


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_fp64_matches_reference_golden(name):
    """Fields, NTFF accumulators, and where the case has them the far-field
    spectrum (ntff*_TimeOutput) and frequency NTFF (ntffTM_Frequency)."""
    ref = dict(np.load(GOLDEN / f"{name}.npz"))
    sim, got = run_gpu(name)
    assert float(got["meta_time"]) == float(ref["meta_time"])
    assert sim.array_size == int(ref["meta_array_size"])
    bad = compare(got, ref, TOL)
    assert not bad, f"{name}: {bad}"


def test_gpu_spectrum_rejects_more_than_8192_steps():
    m = _engine()
    sim = m.Simulation("TM_UPML", m.FieldInfo(300, 300, 5, 8, 100, 0, 9000))
    with pytest.raises(m.FdtdError):
        sim.spectrum()


MODEL_CASES = ["mpi_tm_circle", "mpi_te_circle", "mpi_tm_morpho", "mpi_te_morpho_eps225", "ser_tm_circle",
               "ser_te_circle", "mpi_tm_zigzag", "mpi_te_zigzag_40deg", "split_tm_circle", "split_te_circle_30deg",
               "ns_tm_morpho", "ns_te_circle_20deg"]


def _product_model(spec):
    m = _engine()
    if spec[0] == "circle":
        return m.MODEL_CIRCLE, [spec[1], spec[2]]
    if spec[0] == "morpho":
        w, t0, t1, layers, branch, edge, eps = spec[1:8]
        return m.MODEL_MORPHO, [w, t0, t1, layers, branch, edge, eps, 0.0]
    if spec[0] == "zigzag":
        return m.MODEL_ZIGZAG, [float(v) for v in spec[1:5]] + [0.0]
    raise ValueError(spec)


@pytest.mark.parametrize("name", MODEL_CASES)
def test_gpu_model_fill_equals_reference_eps(name):
    """Device evaluators of circleModel.c / morphoScaleModel.c / zigzagModel.c
    give the reference's permittivity bit-for-bit at every staggered point."""
    m = _engine()
    c = CASES[name]
    ref = np.load(GOLDEN / f"{name}.npz")
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]))
    sim.fill_model(*_product_model(c["model"]))
    for w in range(3):
        np.testing.assert_array_equal(sim.eps(w), ref[f"eps{w}"], err_msg=f"{name} eps{w}")


def test_gpu_model_fill_run_matches_golden():
    """fill_model + run reproduces the golden fields (no host permittivity)."""
    m = _engine()
    name = "mpi_tm_morpho"
    c = CASES[name]
    ref = dict(np.load(GOLDEN / f"{name}.npz"))
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]))
    sim.fill_model(*_product_model(c["model"]))
    sim.run(c["steps"])
    for w in range(3):
        assert rel(sim.field(w), ref[f"field{w}"]) <= TOL


def test_gpu_bad_eps_rejected():
    m = _engine()
    sim = m.Simulation("MPI_TM_UPML", m.FieldInfo(300, 320, 5, 6, 100, 0, 150))
    e = np.ones((sim.n_px, sim.n_py))
    e[3, 4] = -1.0
    with pytest.raises(m.FdtdError):
        sim.set_eps(e)


def test_gpu_clock_outside_step_num_rejected():
    m = _engine()
    sim = m.Simulation("MPI_TM_UPML", m.FieldInfo(300, 320, 5, 6, 100, 0, 10))
    sim.run(10)
    with pytest.raises(m.FdtdError):
        sim.run(1)
    with pytest.raises(m.FdtdError):
        sim.update(-1.0, 0.0)
    assert sim.status == 0


@pytest.mark.parametrize("mode,chunk,block", [(0, 1024, 32), (1, 64, 32), (1, 4096, 32), (2, 1024, 1),
                                              (2, 1024, 7), (2, 1024, 64)])
def test_gpu_ntff_variants_agree(mode, chunk, block):
    """Direct-atomic, shared-window and time-blocked NTFF deposits agree with
    the golden rows (block 7 leaves a partial block and crosses binades of the
    retarded time inside blocks, which takes the exact per-step path)."""
    m = _engine()
    name = "mpi_tm_discs_30deg"
    c = CASES[name]
    ref = dict(np.load(GOLDEN / f"{name}.npz"))
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]))
    sim.set_option(m.OPT_NTFF_MODE, mode)
    sim.set_option(m.OPT_NTFF_CHUNK, chunk)
    sim.set_option(m.OPT_NTFF_BLOCK, block)
    sim.set_eps(*_eps_for(name, c))
    sim.run(c["steps"])
    got = capture([sim.field(w) for w in range(3)], [sim.eps(w) for w in range(3)],
                  [sim.ntff(w) for w in range(3)], sim.array_size, "full")
    bad = compare(got, {k: v for k, v in ref.items() if k.startswith("ntff")}, TOL)
    assert not bad, bad
    assert sim.status == 0


@pytest.mark.parametrize("rows", [2, 4, 8])
@pytest.mark.parametrize("name", ["mpi_tm_discs_30deg", "mpi_te_discs_60deg", "ser_tm_circle"])
def test_gpu_rows_per_thread_variants(name, rows):
    """Every rows-per-thread setting of the stencil kernels gives the golden fields."""
    m = _engine()
    c = CASES[name]
    ref = dict(np.load(GOLDEN / f"{name}.npz"))
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]))
    sim.set_option(m.OPT_ROWS, rows)
    sim.set_eps(*_eps_for(name, c))
    sim.run(c["steps"])
    for w in range(3):
        assert rel(sim.field(w), ref[f"field{w}"]) <= TOL, (name, rows, w)


def test_gpu_fp32_error_against_fp64():
    """FP32 fields with FP64 NTFF: field relative L2 and far-field error (dB)
    against the FP64 engine on the 1044^2 Mie case (r 500 nm, eps 2.25)."""
    from mpifdtd_gb300.precision import compare_precisions
    m = _engine()
    fi = m.FieldInfo(5220, 5220, 5, 10, 500, 0, 4000)
    rep = compare_precisions("MPI_TM_UPML", fi, (m.MODEL_CIRCLE, [500.0, 2.25]), steps=600)
    assert rep["field_rel_l2"]["Ez"] < 1e-4, rep
    assert rep["ntff_rel_l2"] < 1e-4, rep
    assert rep["farfield_db_max"] < 0.01, rep


def test_gpu_vacuum_config1_exact_zero():
    """The 276^2 vacuum run (2000 steps): every output stays exactly 0."""
    _, got = run_gpu("mpi_tm_vacuum_c1")
    for k, v in got.items():
        if not k.startswith("meta_"):
            assert np.all(np.asarray(v) == 0), k


@pytest.mark.parametrize("solver", ["MPI_TM_UPML", "MPI_TE_UPML"])
def test_gpu_fp64_matches_oracle_full_c2_grid(solver):
    """1044^2 Mie cylinder (r 500 nm, eps 2.25), 120 steps: full arrays."""
    from oracle.pyoracle import FieldInfo as OFI, Model, OracleSim
    m = _engine()
    fi = (5220, 5220, 5, 10, 500, 0, 4000)
    o = OracleSim(solver, OFI(*fi), Model.circle(500, 2.25))
    sim = m.Simulation(solver, m.FieldInfo(*fi))
    sim.set_eps(*[o.eps(w)[1:-1, 1:-1] for w in range(3)])
    steps = 120
    o.step(steps)
    sim.run(steps)
    for w in range(3):
        e = rel(sim.field(w), o.field(w)[1:-1, 1:-1])
        assert e <= TOL, (solver, "field", w, e)
        e = rel(sim.ntff(w), o.ntff(w))
        assert e <= TOL, (solver, "ntff", w, e)


def test_gpu_drop_in_update_clock_matches_run():
    """fdtd_update(time, ray_coef) driven by a host clock (simulator_calc +
    field_nextStep, simulator.c:247-251) equals fdtd_run."""
    m = _engine()
    fi = m.FieldInfo(300, 320, 5, 6, 100, 0, 150)
    eps = _eps_for("mpi_tm_circle", CASES["mpi_tm_circle"])
    a = m.Simulation("MPI_TM_UPML", fi)
    b = m.Simulation("MPI_TM_UPML", fi)
    a.set_eps(*eps)
    b.set_eps(*eps)
    a.run(60)
    t, rc = 0.0, 0.0
    for _ in range(60):
        b.update(t, rc)
        t += 1.0
        rc = 1.0 - np.exp(-(0.01 * t) ** 2)
    for w in range(3):
        assert rel(b.field(w), a.field(w)) <= 1e-15
        assert rel(b.ntff(w), a.ntff(w)) <= 1e-15


def test_gpu_reset_zeroes_fields():
    m = _engine()
    fi = m.FieldInfo(300, 320, 5, 6, 100, 0, 150)
    sim = m.Simulation("MPI_TE_UPML", fi)
    sim.set_eps(*_eps_for("mpi_te_circle", CASES["mpi_te_circle"]))
    sim.run(30)
    assert np.abs(sim.field(1)).max() > 0
    sim.reset()
    assert sim.time == 0
    for w in range(3):
        assert np.all(sim.field(w) == 0)


def test_gpu_ntff_guards_untouched():
    sim, _ = run_gpu("mpi_tm_circle")
    for w in range(3):
        assert np.all(sim.ntff_guard(w) == 0)


def test_gpu_split_and_ns_solvers_refuse_ntff_and_fp32():
    """The split-field / NS solvers have no NTFF and run in FP64 only."""
    m = _engine()
    fi = m.FieldInfo(300, 300, 5, 10, 100, 0, 20)
    with pytest.raises(m.FdtdError):
        m.Simulation("TM_2D", fi, "f32")
    sim = m.Simulation("NS_TM_2D", fi)
    sim.run(5)
    for call in (sim.frequency, sim.spectrum, lambda: sim.ntff(0)):
        with pytest.raises(m.FdtdError):
            call()
    ez, ezx, ezy = sim.field(0), sim.field(3), sim.field(4)
    np.testing.assert_array_equal(ez, ezx + ezy)            # nsFdtdTM.c:73-76: Ez = Ezx + Ezy


def test_gpu_flush_deposits_a_run_shorter_than_the_ntff_block():
    """A run of fewer steps than the time-blocked NTFF buffer (32 steps)
    leaves its deposit pending; fdtd_flush enqueues it on the engine stream,
    the profiler counts it as NTFF deposit time, and the accumulators then
    hold every step (mpiTM_UPML.c:196-217 deposits inside each update())."""
    m = _engine()
    fi = m.FieldInfo(300, 320, 5, 6, 100, 0, 150)
    eps = _eps_for("mpi_tm_circle", CASES["mpi_tm_circle"])
    a = m.Simulation("MPI_TM_UPML", fi)
    b = m.Simulation("MPI_TM_UPML", fi)
    for s in (a, b):
        s.set_eps(*eps)
        s.run(40)                       # past the source ramp: the path carries field
        s.synchronize()
    a.profile(True)
    a.run(20)
    a.flush()
    prof = a.profile_read()
    a.profile(False)
    assert prof["steps"] == 20
    assert prof["ntff_deposit"] > 0
    b.set_option(m.OPT_NTFF_MODE, 0)    # direct per-step deposit as the reference does
    b.run(20)
    for w in range(3):
        assert rel(a.ntff(w), b.ntff(w)) <= 1e-12


SETTINGS = {"c05_cubic_inset20": dict(courant=0.5, pml_order=3, ntff_inset=20),
            "c06_quartic_inset8": dict(courant=0.6, pml_order=4, ntff_inset=8)}


@pytest.mark.parametrize("setting", sorted(SETTINGS))
@pytest.mark.parametrize("solver", ["MPI_TM_UPML", "MPI_TE_UPML", "TM_UPML", "TE_UPML"])
def test_gpu_settings_the_reference_fixes_match_oracle(solver, setting):
    """Courant number, sigma grading order and NTFF inset away from the
    reference's hard-coded values (field.h:70, field.c:259-283,
    field.c:136-139): fields, NTFF accumulators and the far field (frequency
    NTFF of the MPI solvers, spectrum of the serial ones) against the oracle
    restatement at the same settings, 1e-12."""
    m = _engine()
    from oracle.pyoracle import FieldInfo as OFI, Model, OracleSim
    fi = (500, 520, 5, 8, 120, 20, 150)
    o = OracleSim(solver, OFI(*fi, **SETTINGS[setting]), Model.circle(90, 2.25))
    mpi = solver.startswith("MPI")
    sim = m.Simulation(solver, m.FieldInfo(*fi, **SETTINGS[setting]))
    sim.set_eps(*[crop(o.eps(w), mpi) for w in range(3)])
    assert (sim.geo.ntff_left, sim.array_size) == (o.left, o.array_size)
    o.step(150)
    sim.run(150)
    for w in range(3):
        e = rel(sim.field(w), crop(o.field(w), mpi))
        assert e <= TOL, (solver, setting, "field", w, e)
        e = rel(sim.ntff(w), o.ntff(w))
        assert e <= TOL, (solver, setting, "ntff", w, e)
    if mpi:
        e = rel(sim.frequency(), o.frequency())
    else:
        e = rel(sim.spectrum(), o.time_output())
    assert e <= TOL, (solver, setting, "far field", e)


@pytest.mark.parametrize("solver", ["MPI_TM_UPML", "MPI_TE_UPML"])
def test_gpu_settings_blocked_kernels_match_oracle(solver):
    """The temporally blocked kernels (K = 4) at a Courant number of 0.5,
    cubic grading and a 20-cell NTFF inset."""
    m = _engine()
    from oracle.pyoracle import FieldInfo as OFI, Model, OracleSim
    fi = (500, 520, 5, 8, 120, 0, 150)
    st = SETTINGS["c05_cubic_inset20"]
    o = OracleSim(solver, OFI(*fi, **st), Model.circle(90, 2.25))
    sim = m.Simulation(solver, m.FieldInfo(*fi, **st))
    sim.set_eps(*[crop(o.eps(w), True) for w in range(3)])
    sim.set_option(m.OPT_TBLOCK, 4)
    o.step(120)
    sim.run(120)
    for w in range(3):
        assert rel(sim.field(w), crop(o.field(w), True)) <= TOL
        assert rel(sim.ntff(w), o.ntff(w)) <= TOL
