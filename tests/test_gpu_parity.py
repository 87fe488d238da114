"""GPU parity: the CUDA engine against the reference's golden vectors and the oracle.

Bar (the benchmark spec): FP64 fields and NTFF accumulators within 1e-12 relative L2
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
    ntff = [sim.ntff(w) for w in range(3)]
    out = capture(fields, eps, ntff, sim.array_size, c["kind"], c.get("rows", "all"))
    out["meta_time"] = np.array(sim.time)
    return sim, out


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_fp64_matches_reference_golden(name):
    ref = dict(np.load(GOLDEN / f"{name}.npz"))
    sim, got = run_gpu(name)
    assert float(got["meta_time"]) == float(ref["meta_time"])
    assert sim.array_size == int(ref["meta_array_size"])
    skip = {"spectrum", "frequency"}
    bad = compare(got, {k: v for k, v in ref.items() if k not in skip}, TOL)
    assert not bad, f"{name}: {bad}"


def test_gpu_vacuum_config1_exact_zero():
    """SURVEY config 1 (276^2, vacuum, 2000 steps): every output stays exactly 0."""
    _, got = run_gpu("mpi_tm_vacuum_c1")
    for k, v in got.items():
        if not k.startswith("meta_"):
            assert np.all(np.asarray(v) == 0), k


@pytest.mark.parametrize("solver", ["MPI_TM_UPML", "MPI_TE_UPML"])
def test_gpu_fp64_matches_oracle_full_c2_grid(solver):
    """1044^2 Mie cylinder (SURVEY config 2 grid, eps 2.25), 120 steps: full arrays."""
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
