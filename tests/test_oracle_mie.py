"""Known-answer physics check of the oracle's CW path: the far field of a
dielectric cylinder against the Mie series (oracle/mie.py).

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
