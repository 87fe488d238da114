"""Broadband batch (fdtd_batch_broadband): the reference's Gaussian pulse
(field.c:224-256) drives every instance and a running DFT of the NTFF path
gives the far field at many wavelengths from one run.

No reference test covers this path (the reference's broadband run is one
serial solver per structure with an 8192-point FFT); it is pinned by physics:
the Mie series of a dielectric cylinder at seven wavelengths from one run, and
the CW engine's own far field at the carrier wavelength.  The time-domain
NTFF's angle a is the direction a (its kernel is e^{-i k r.r'}).
"""
import numpy as np
import pytest

from oracle import mie

pytestmark = pytest.mark.gpu

LAMS = [400, 450, 500, 550, 600, 650, 700]
FI = (800, 800, 5, 10, 500, 0, 1600)   # 160^2 cells of 5 nm, 10-cell UPML, carrier 500 nm


def _broadband(precision, radii=(100.0, 150.0), eps=2.25, k=4, stride=None):
    import mpifdtd_gb300 as m
    b = m.Batch("MPI_TM_UPML", [m.FieldInfo(*FI) for _ in radii], precision, no_time_ntff=False)
    b.set_option(m.OPT_TBLOCK, k)
    if stride is not None:
        b.set_option(m.OPT_DFT_STRIDE, stride)
    for s, r in zip(b.instances, radii):
        s.fill_model(m.MODEL_CIRCLE, [r, eps])
    b.broadband(LAMS)
    b.run()
    out = list(b.broadband_spectra())
    for i in range(len(radii)):   # the batched read-out equals the per-instance one
        np.testing.assert_array_equal(out[i], b.broadband_spectrum(i))
    assert all(s.status == 0 for s in b.instances)
    b.close()
    return out


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_broadband_far_field_matches_mie_at_seven_wavelengths(precision):
    """Cylinders r = 100, 150 nm, eps 2.25: the intensity pattern at every
    wavelength from 400 to 700 nm is within 3 % (relative L2 after one scale)
    of the series, and the scattering is forward (the forward lobe of these
    small cylinders is flat to 0.1 % over a few degrees, so the test takes
    the intensity at 0 degrees against the maximum, not the arg max)."""
    out = _broadband(precision)
    for r, inten in zip((100.0, 150.0), out):
        for k, lam in enumerate(LAMS):
            ref = np.abs(mie.far_field(r, lam, 2.25, "TM", angles_deg=np.arange(360))) ** 2
            err, _ = mie.pattern_error(inten[k], ref)
            assert err < 0.03, (r, lam, err)
            assert inten[k][0] >= 0.99 * inten[k].max() and inten[k][0] > 2 * inten[k][180], (r, lam)


def test_broadband_dft_of_every_sixteenth_step_equals_every_step():
    """The batch samples its DFT every FDTD_OPT_DFT_STRIDE steps (16 by
    default); with K = 1 and stride 1 it samples every step.  The pulse's
    spectrum is far below the sampled series' Nyquist frequency, so both give
    the same far fields (FP64 fields), and so does stride 4."""
    every = _broadband("f64", k=1, stride=1)
    for x, y in zip(_broadband("f64", k=4), every):
        assert np.linalg.norm(x - y) / np.linalg.norm(y) < 1e-4
    for x, y in zip(_broadband("f64", k=4, stride=4), every):
        assert np.linalg.norm(x - y) / np.linalg.norm(y) < 1e-4


def test_broadband_fp32_fields_agree_with_fp64():
    a64, a32 = _broadband("f64"), _broadband("f32")
    for x, y in zip(a32, a64):
        assert np.linalg.norm(x - y) / np.linalg.norm(y) < 1e-4


def test_broadband_equals_cw_steady_state_at_the_carrier():
    """The CW engine's frequency-domain far field (ntffTM_Frequency of the
    final fields after 30 periods; angle a is direction a + 180) and the
    broadband run at the carrier wavelength give the same pattern."""
    import mpifdtd_gb300 as m
    bb = _broadband("f64", radii=(150.0,))[0][LAMS.index(500)]
    steps = int(np.ceil(30 * (500 / 5) / 0.7071))
    sim = m.Simulation("MPI_TM_UPML", m.FieldInfo(800, 800, 5, 10, 500, 0, steps))
    sim.fill_model(m.MODEL_CIRCLE, [150.0, 2.25])
    sim.run(steps)
    cw = np.roll(np.abs(sim.frequency()) ** 2, 180)
    err, _ = mie.pattern_error(bb, cw)
    assert err < 0.02, err


def test_broadband_rejects_te_and_missing_ntff_path():
    import mpifdtd_gb300 as m
    fi = m.FieldInfo(*FI)
    b = m.Batch("MPI_TE_UPML", [fi], "f32", no_time_ntff=False)
    with pytest.raises(m.FdtdError):
        b.broadband(LAMS)
    b.close()
    b = m.Batch("MPI_TM_UPML", [fi], "f32", no_time_ntff=True)
    with pytest.raises(m.FdtdError):
        b.broadband(LAMS)
    b.close()


def test_broadband_far_field_does_not_depend_on_the_batch_around_it():
    """Instances of one configuration share a far-field launch (groups of up
    to 16 maps over one path); an instance's spectrum is the same alone, in a
    batch of 20 with a second configuration interleaved, and in any group
    position."""
    import mpifdtd_gb300 as m
    other = (900, 900, 5, 10, 500, 0, 1600)
    cfgs = [FI if q % 3 else other for q in range(20)]
    radii = [90.0 + 4 * q for q in range(20)]

    def run(fis, rs):
        b = m.Batch("MPI_TM_UPML", [m.FieldInfo(*f) for f in fis], "f32", no_time_ntff=False)
        b.set_option(m.OPT_TBLOCK, 4)
        for s, r in zip(b.instances, rs):
            s.fill_model(m.MODEL_CIRCLE, [r, 2.25])
        b.broadband(LAMS)
        b.run()
        out = b.broadband_spectra()
        b.close()
        return out

    mixed = run(cfgs, radii)
    for q in (0, 1, 2, 17, 19):
        alone = run([cfgs[q]], [radii[q]])[0]
        np.testing.assert_array_equal(mixed[q], alone)
