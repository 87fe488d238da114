"""Temporally blocked stepping (FDTD_OPT_TBLOCK): K steps per pass over HBM.

The blocked kernels compute the same cell updates as the one-step kernels in
the same order, so the FP64 results meet the same 1e-12 bar against the
reference's golden vectors; FP32 blocked runs are compared with FP32 one-step
runs (same arithmetic, so agreement to a few FP32 ulps of the field norm).
"""
import numpy as np
import pytest

from tests.golden.cases import CASES
from tests.golden.golden_io import capture, compare, rel
from tests.test_gpu_parity import _eps_for

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _engine():
    import mpifdtd_gb300 as m
    return m


def _golden(name):
    from tests.test_gpu_parity import GOLDEN
    return dict(np.load(GOLDEN / f"{name}.npz"))


def _run(name, precision="f64", k=0, rows=0, split=None, ntff_block=None):
    m = _engine()
    c = CASES[name]
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]), precision)
    if ntff_block:
        sim.set_option(m.OPT_NTFF_BLOCK, ntff_block)
    sim.set_option(m.OPT_TBLOCK, k)
    sim.set_option(m.OPT_TBLOCK_ROWS, rows)
    sim.set_eps(*_eps_for(name, c))
    steps = c["steps"]
    for n in (split or [steps]):
        sim.run(n)
    return sim


MPI_CASES = ["mpi_tm_circle", "mpi_te_circle", "mpi_tm_morpho", "mpi_tm_discs_30deg", "mpi_te_discs_60deg"]


@pytest.mark.parametrize("k,rows", [(1, 0), (2, 7), (4, 0), (4, 5), (2, 64)])
@pytest.mark.parametrize("name", MPI_CASES)
def test_tblock_fp64_matches_reference_golden(name, k, rows):
    """Fields and NTFF accumulators of blocked runs against the golden vectors
    (tile heights 5 and 7 put segment seams inside the NTFF path and the PML)."""
    c = CASES[name]
    sim = _run(name, k=k, rows=rows)
    got = capture([sim.field(w) for w in range(3)], [sim.eps(w) for w in range(3)],
                  [sim.ntff(w) for w in range(3)], sim.array_size, c["kind"], c.get("rows", "all"))
    ref = _golden(name)
    bad = compare(got, {key: v for key, v in ref.items() if key.startswith(("field", "ntff"))}, TOL)
    assert not bad, (name, k, rows, bad)
    assert sim.status == 0


def test_tblock_mixed_update_run_and_odd_ntff_block():
    """Single steps through fdtd_update, then blocked runs whose step counts are
    not multiples of K, with an NTFF deposit block (7) that K (4) does not divide."""
    m = _engine()
    name = "mpi_tm_discs_30deg"
    c = CASES[name]
    ref = _golden(name)
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]))
    sim.set_option(m.OPT_NTFF_BLOCK, 7)
    sim.set_option(m.OPT_TBLOCK, 4)
    sim.set_eps(*_eps_for(name, c))
    steps = c["steps"]
    t, rc = 0.0, 0.0
    for _ in range(3):
        sim.update(t, rc)
        t += 1.0
        rc = 1.0 - np.exp(-(0.01 * t) ** 2)
    sim.time = t  # the host clock of the drop-in path, handed back to fdtd_run
    rest = steps - 3
    sim.run(rest // 2 + 1)
    sim.run(rest - (rest // 2 + 1))
    got = capture([sim.field(w) for w in range(3)], [sim.eps(w) for w in range(3)],
                  [sim.ntff(w) for w in range(3)], sim.array_size, "full")
    bad = compare(got, {key: v for key, v in ref.items() if key.startswith(("field", "ntff"))}, TOL)
    assert not bad, bad


@pytest.mark.parametrize("solver", ["MPI_TM_UPML", "MPI_TE_UPML"])
def test_tblock_fp64_matches_oracle_c2_grid(solver):
    """1044^2 Mie cylinder: interior tiles (no PML in the cone) and PML tiles
    both run; full arrays against the oracle."""
    from oracle.pyoracle import FieldInfo as OFI, Model, OracleSim
    m = _engine()
    fi = (5220, 5220, 5, 10, 500, 0, 4000)
    o = OracleSim(solver, OFI(*fi), Model.circle(500, 2.25))
    eps = [o.eps(w)[1:-1, 1:-1] for w in range(3)]
    steps = 120
    o.step(steps)
    for k, rows in ((4, 0), (2, 48)):
        sim = m.Simulation(solver, m.FieldInfo(*fi))
        sim.set_eps(*eps)
        sim.set_option(m.OPT_TBLOCK, k)
        sim.set_option(m.OPT_TBLOCK_ROWS, rows)
        sim.run(steps)
        for w in range(3):
            e = rel(sim.field(w), o.field(w)[1:-1, 1:-1])
            assert e <= TOL, (solver, k, "field", w, e)
            e = rel(sim.ntff(w), o.ntff(w))
            assert e <= TOL, (solver, k, "ntff", w, e)


@pytest.mark.parametrize("solver", ["MPI_TM_UPML", "MPI_TE_UPML"])
@pytest.mark.parametrize("k,cols", [(1, 1), (2, 1), (4, 1), (8, 1), (2, 2), (4, 2)])
def test_tblock_fp32_equals_fp32_one_step(solver, k, cols):
    m = _engine()
    fi = m.FieldInfo(5220, 5220, 5, 10, 500, 0, 4000)
    sims = []
    for kk in (0, k):
        s = m.Simulation(solver, fi, "f32")
        s.fill_model(m.MODEL_CIRCLE, [500.0, 2.25])
        s.set_option(m.OPT_TBLOCK, kk)
        s.set_option(m.OPT_TBLOCK_COLS, cols)
        s.set_option(m.OPT_TBLOCK_ROWS, 48 if cols == 2 else 0)
        s.run(200)
        sims.append(s)
    # same cell arithmetic; the kernels differ only in FMA contraction, so FP32
    # rounding over 200 steps stays within ~80 ulps of the field norm
    for w in range(3):
        assert rel(sims[1].field(w), sims[0].field(w)) < 5e-6, (solver, k, w)
        assert rel(sims[1].ntff(w), sims[0].ntff(w)) < 5e-6, (solver, k, w)


def test_autotune_keeps_state_and_picks_a_valid_setting():
    m = _engine()
    name = "mpi_tm_morpho"
    c = CASES[name]
    ref = _golden(name)
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]))
    sim.set_eps(*_eps_for(name, c))
    half = c["steps"] // 2
    sim.run(half)
    before = [sim.field(w) for w in range(3)]
    res = sim.autotune()
    assert res["tblock"] in (0, 1, 2, 4) and res["stencil_ms_per_step"] > 0
    assert sim.get_option(m.OPT_TBLOCK) == res["tblock"]
    for w in range(3):
        np.testing.assert_array_equal(sim.field(w), before[w])
    sim.run(c["steps"] - half)
    for w in range(3):
        assert rel(sim.field(w), ref[f"field{w}"]) <= TOL


def test_tblock_rejects_split_ns_solvers_and_bad_depths():
    m = _engine()
    for solver in ("TM_2D", "NS_TE_2D"):               # split-field / NS: one step per launch
        s = m.Simulation(solver, m.FieldInfo(300, 300, 5, 8, 100, 0, 100))
        with pytest.raises(m.FdtdError):
            s.set_option(m.OPT_TBLOCK, 2)
    s = m.Simulation("TM_UPML", m.FieldInfo(300, 300, 5, 8, 100, 0, 100), "f32")
    with pytest.raises(m.FdtdError):
        s.set_option(m.OPT_TBLOCK, 8)                  # serial solvers: K = 1, 2, 4
    s = m.Simulation("MPI_TM_UPML", m.FieldInfo(300, 300, 5, 8, 100, 0, 100))
    with pytest.raises(m.FdtdError):
        s.set_option(m.OPT_TBLOCK, 8)
    with pytest.raises(m.FdtdError):
        s.set_option(m.OPT_TBLOCK, 3)
    with pytest.raises(m.FdtdError):
        s.set_option(m.OPT_TBLOCK_COLS, 2)   # FP64 fields


# ---- the serial solvers (fdtdTM_upml.c:54-66, fdtdTE_upml.c:168-192): H half-step first, Gaussian pulse

SERIAL_CASES = ["ser_tm_circle", "ser_te_circle"]


@pytest.mark.parametrize("k,rows", [(1, 0), (2, 7), (4, 0), (4, 5), (2, 64)])
@pytest.mark.parametrize("name", SERIAL_CASES)
def test_tblock_serial_fp64_matches_reference_golden(name, k, rows):
    """Fields, NTFF accumulators and the far-field spectrum (ntff*_TimeOutput)
    of blocked serial runs against the reference's own serial solvers; the
    TE case (20 degrees) drives both E components with the pulse."""
    c = CASES[name]
    sim = _run(name, k=k, rows=rows)
    launches_blocked = sim.launches
    got = capture([sim.field(w) for w in range(3)], [sim.eps(w) for w in range(3)],
                  [sim.ntff(w) for w in range(3)], sim.array_size, c["kind"], c.get("rows", "all"))
    got["spectrum"] = sim.spectrum()
    ref = _golden(name)
    bad = compare(got, {key: v for key, v in ref.items() if key.startswith(("field", "ntff", "spectrum"))}, TOL)
    assert not bad, (name, k, rows, bad)
    assert sim.status == 0
    one = _run(name, k=0)
    if k > 1:   # the blocked kernels ran: fewer launches than one step at a time
        assert launches_blocked < one.launches, (launches_blocked, one.launches)


@pytest.mark.parametrize("solver,angle", [("TM_UPML", 0), ("TE_UPML", 30), ("TE_UPML", 0)])
@pytest.mark.parametrize("k,cols", [(1, 1), (2, 1), (4, 1), (2, 2), (4, 2)])
def test_tblock_serial_fp32_equals_fp32_one_step(solver, angle, k, cols):
    """1044^2 Mie cylinder, pulse source, interior and PML tiles: FP32 blocked
    against FP32 one-step (same cell arithmetic up to FMA contraction; at 0
    degrees the tiles read the pulse from per-row tables)."""
    m = _engine()
    fi = m.FieldInfo(5220, 5220, 5, 10, 500, angle, 1200)
    sims = []
    for kk in (0, k):
        s = m.Simulation(solver, fi, "f32")
        s.fill_model(m.MODEL_CIRCLE, [500.0, 2.25])
        s.set_option(m.OPT_TBLOCK, kk)
        s.set_option(m.OPT_TBLOCK_COLS, cols)
        s.set_option(m.OPT_TBLOCK_ROWS, 48 if cols == 2 else 0)
        s.run(700)            # the pulse reaches the cylinder after ~500 steps
        sims.append(s)
    for w in range(3):
        assert rel(sims[1].field(w), sims[0].field(w)) < 5e-6, (solver, k, w)
        assert rel(sims[1].ntff(w), sims[0].ntff(w)) < 5e-6, (solver, k, w)
    assert np.abs(sims[0].field(0)).max() > 0


def test_tblock_serial_runs_split_across_calls_and_updates():
    """A serial run through fdtd_update steps, then blocked runs whose lengths
    K does not divide, ends where the reference's run does."""
    m = _engine()
    name = "ser_tm_circle"
    c = CASES[name]
    ref = _golden(name)
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]))
    sim.set_option(m.OPT_NTFF_BLOCK, 7)
    sim.set_option(m.OPT_TBLOCK, 4)
    sim.set_eps(*_eps_for(name, c))
    t = 0.0
    for _ in range(3):
        sim.update(t, 0.0)
        t += 1.0
    sim.time = t
    rest = c["steps"] - 3
    sim.run(rest // 2 + 1)
    sim.run(rest - (rest // 2 + 1))
    got = capture([sim.field(w) for w in range(3)], [sim.eps(w) for w in range(3)],
                  [sim.ntff(w) for w in range(3)], sim.array_size, c["kind"], c.get("rows", "all"))
    bad = compare(got, {key: v for key, v in ref.items() if key.startswith(("field", "ntff"))}, TOL)
    assert not bad, bad


def test_autotune_serial_solver_keeps_state_and_picks_a_valid_setting():
    """The autotuner times the serial solvers' own order (H half-step first,
    pulse) and leaves the fields as they were; the run it tunes still meets
    the golden vectors."""
    m = _engine()
    name = "ser_te_circle"
    c = CASES[name]
    ref = _golden(name)
    sim = m.Simulation(c["solver"], m.FieldInfo(*c["fi"]))
    sim.set_eps(*_eps_for(name, c))
    half = c["steps"] // 2
    sim.run(half)
    before = [sim.field(w) for w in range(3)]
    res = sim.autotune()
    assert res["tblock"] in (0, 1, 2, 4) and res["stencil_ms_per_step"] > 0
    assert all(k != 8 for k, _, _, _ in res["candidates"])
    for w in range(3):
        np.testing.assert_array_equal(sim.field(w), before[w])
    sim.run(c["steps"] - half)
    for w in range(3):
        assert rel(sim.field(w), ref[f"field{w}"]) <= TOL
