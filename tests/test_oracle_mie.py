"""Known-answer physics check of the oracle's CW path: the far field and the
1.2-lambda near-field ring of a dielectric cylinder against the Mie series
(oracle/mie.py).

The MPI UPML solvers (scatteredWave source, mpiTM_UPML.c:337-374 /
mpiTE_UPML.c:250-281) run a cylinder to steady state and the frequency-domain
NTFF (ntffTM.c:72-158 / ntffTE.c:242-338) gives the far field; its intensity
pattern matches the series' |T(phi + 180)|^2 up to the solver's own scale
(angle a of the NTFF is the direction a + 180 degrees of the series'
e^{-i w t} convention).  This pins the TE frequency restatement, which no
reference test or caller exercises, by physics instead of by a golden vector.
"""
import numpy as np
import pytest

from oracle import mie
from oracle import pyoracle as po


def test_series_is_lossless_and_symmetric():
    """Optical theorem per order for a real index: Re b_n = -|b_n|^2, and b_-n = b_n."""
    for pol in ("TM", "TE"):
        for x, m in ((0.5, 1.2), (3.0, 1.5), (12.0, 2.0)):
            n, b = mie.coefficients(x, m, pol)
            assert np.abs(b.real + np.abs(b) ** 2).max() < 1e-12
            assert np.abs(b - b[::-1]).max() < 1e-12
            assert np.abs(b[[0, -1]]).max() < 1e-12      # the order bound is enough


def test_series_rejects_unknown_polarisation():
    with pytest.raises(ValueError):
        mie.coefficients(1.0, 1.5, "TEM")


@pytest.mark.parametrize("solver,pol", [("MPI_TM_UPML", "TM"), ("MPI_TE_UPML", "TE")])
def test_oracle_far_field_matches_mie_series(solver, pol):
    """r = 100 nm, eps = 2.25, lambda = 300 nm on 5 nm cells, 900 steps: the
    intensity pattern is within 2 % (relative L2) of the series."""
    r, lam, eps = 100, 300, 2.25
    sim = po.OracleSim(solver, po.FieldInfo(800, 800, 5, 10, lam, 0, 900), po.Model.circle(r, eps))
    sim.step(900)
    inten = np.abs(sim.frequency()) ** 2
    ref = np.abs(mie.far_field(r, lam, eps, pol, angles_deg=np.arange(360) + 180)) ** 2
    err, _ = mie.pattern_error(inten, ref)
    assert err < 0.02, err
    assert abs(int(np.argmax(inten)) - 180) <= 2   # forward scattering of the +x plane wave


@pytest.mark.parametrize("solver,pol", [("TM_2D", "TM"), ("NS_TM_2D", "TM"), ("TE_2D", "TE"), ("NS_TE_2D", "TE"),
                                        ("MPI_TM_UPML", "TM")])
def test_oracle_elliptic_ring_matches_mie_near_field(solver, pol):
    """field_outputElliptic's ring (|E|^2 of the scattered field at 1.2 lambda,
    Ez for TM, Ey for TE) of every solver family against the series, in
    absolute amplitude: r = 150 nm, eps = 2.25, lambda = 300 nm, 1000 steps."""
    from oracle import outputs
    r, lam, eps = 150, 300, 2.25
    sim = po.OracleSim(solver, po.FieldInfo(1200, 1200, 5, 10, lam, 0, 1000), po.Model.circle(r, eps))
    sim.step(1000)
    f = sim.field(0 if pol == "TM" else 1)
    if sim.mpi:
        f = f[1:-1, 1:-1]
    ring = outputs.elliptic_ring(f, lam / 5)
    ref = mie.near_field_ring(r, lam, eps, pol, 1.2 * lam)
    err = float(np.linalg.norm(ring - ref) / np.linalg.norm(ref))
    assert err < (0.02 if pol == "TM" else 0.04), err


@pytest.mark.parametrize("solver,pol", [("MPI_TM_UPML", "TM"), ("MPI_TE_UPML", "TE")])
def test_oracle_far_field_matches_mie_with_settings_the_reference_fixes(solver, pol):
    """The restatement with a Courant number of 0.5, cubic sigma grading and
    the NTFF path 20 cells inside the PML -- settings the reference hard-codes
    (field.h:70, field.c:259-283, field.c:136-139) and so cannot produce golden
    vectors for -- still lands on the Mie series: same cylinder as above, run
    1.41x longer since a step now advances the wave 0.5 cells instead of 0.7071."""
    r, lam, eps = 100, 300, 2.25
    fi = po.FieldInfo(800, 800, 5, 10, lam, 0, 1300, courant=0.5, pml_order=3, ntff_inset=20)
    sim = po.OracleSim(solver, fi, po.Model.circle(r, eps))
    assert (sim.left, sim.bottom) == (30, 30) and sim.right == 160 - 30
    sim.step(1300)
    inten = np.abs(sim.frequency()) ** 2
    ref = np.abs(mie.far_field(r, lam, eps, pol, angles_deg=np.arange(360) + 180)) ** 2
    err, _ = mie.pattern_error(inten, ref)
    assert err < 0.02, err
    assert abs(int(np.argmax(inten)) - 180) <= 2
