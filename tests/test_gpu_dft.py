"""Running-DFT NTFF (fdtd_dft_*): validated against the time-domain pipeline.

(1) The algebra: the DFT's far field equals the Fourier sum of the engine's
own time-domain accumulators (pinned to the reference) over all bins, up to
rounding, except at the few corner angles whose last deposits the flat
[360][arraySize] index books into the neighbouring angle's row (the time
domain's spill, which a per-angle DFT does not reproduce).
(2) The reference's output: the spectrum of ntff*_TimeOutput transforms only
the first step_num bins; once the pulse has left the NTFF box the DFT
spectrum agrees with it (here to 1e-5 relative L2).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Z0, C = 1.41422712488, 0.7071
LAMS = list(range(380, 701, 40))


def _host_far_field(sim, lams):
    AS = sim.array_size
    U = [sim.ntff(w).reshape(360, AS) for w in range(3)]
    coef = (1 / (4 * math.pi * C)) * np.sqrt(complex(2 * math.pi * C, 0) / complex(0, sim.geo.omega_s))
    mm = np.arange(AS)
    X = np.zeros((360, 2 * len(lams)), complex)
    for a in range(360):
        phi = a * (math.pi / 180.0)
        px, py, sz = -math.sin(phi), math.cos(phi), -1.0
        g = (-px, -py, -Z0 * sz) if sim.tm else (-Z0 * px, -Z0 * py, sz)
        eth = g[0] * U[0][a] + g[1] * U[1][a] + g[2] * U[2][a]
        for l, lam in enumerate(lams):
            idx = math.floor(C * sim.fi.h_u_nm * 8192 / lam)
            for b in (0, 1):
                X[a, 2 * l + b] = coef * np.sum(eth * np.exp(1j * 2 * math.pi * (idx + b) / 8192 * mm))
    return X


def _run(solver, fi, angle_model=(60.0, 2.25)):
    import mpifdtd_gb300 as m
    sim = m.Simulation(solver, m.FieldInfo(*fi))
    sim.fill_model(m.MODEL_CIRCLE, list(angle_model))
    sim.dft_enable(LAMS)
    sim.run(fi[6])
    return sim


@pytest.mark.parametrize("solver,fi", [("TM_UPML", (400, 400, 5, 8, 500, 0, 600)),
                                       ("TE_UPML", (400, 400, 5, 8, 500, 30, 600)),
                                       ("MPI_TM_UPML", (400, 400, 5, 8, 500, 0, 600))])
def test_dft_equals_fourier_sum_of_time_domain_accumulators(solver, fi):
    sim = _run(solver, fi)
    Xd = sim.dft_far_field()
    Xh = _host_far_field(sim, LAMS)
    per_angle = (np.abs(Xd - Xh) / np.abs(Xh).max(axis=0)).max(axis=1)
    assert np.median(per_angle) < 1e-12, np.median(per_angle)
    assert int((per_angle > 1e-9).sum()) <= 8, np.nonzero(per_angle > 1e-9)   # corner-angle spills
    assert per_angle.max() < 1e-4


def test_dft_spectrum_matches_reference_spectrum_after_the_pulse():
    sim = _run("TM_UPML", (400, 400, 5, 8, 500, 0, 3000))
    ref = np.stack([sim.spectrum()[lam - 380] for lam in LAMS])
    got = sim.dft_spectrum()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5


def test_dft_reset_and_state_errors():
    import mpifdtd_gb300 as m
    sim = _run("TM_UPML", (400, 400, 5, 8, 500, 0, 200))
    assert np.abs(sim.dft_far_field()).max() > 0
    sim.reset()
    assert np.abs(sim.dft_far_field()).max() == 0
    s2 = m.Simulation("MPI_TM_UPML", m.FieldInfo(400, 400, 5, 8, 500, 0, 200), no_time_ntff=True)
    with pytest.raises(m.FdtdError):
        s2.dft_enable(LAMS)
