"""Surrogate pipeline: FDTD-generated data, training, what the network gains
over the method without it, and the audited screening with FDTD fallback."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    from mpifdtd_gb300.surrogate import screen as S
    from mpifdtd_gb300.surrogate.data import Generator
    from mpifdtd_gb300.surrogate.model import FNO
    gen = Generator(group=64)
    maps, inten, _ = S.generate(256, 20261211, gen)
    net = FNO(seed=2)
    S.train(net, maps[:192], inten[:192], steps=800, batch=128, lr=1e-3)
    yield S, gen, net, maps, inten
    gen.close()


def test_network_beats_the_network_free_baseline(trained):
    """Held-out error of the trained network against the best constant
    prediction (the mean far field of the training set)."""
    S, gen, net, maps, inten = trained
    ev = S.evaluate(net, maps[192:], inten[192:], inten[:192])
    assert ev["median"] < 0.5 * ev["baseline_mean_far_field"]["median"], ev


def test_mirror_augmentation_matches_the_physics(trained):
    """y -> -y mirrors the far field phi -> -phi (plane wave along x)."""
    S, gen, net, maps, inten = trained
    mm, mi = S.mirror(maps[:4], inten[:4])
    fm = gen.far_field(mm)
    assert np.median(S.rel_err(fm, mi)) < 0.02


def test_translation_augmentation_matches_the_physics(trained):
    """A structure translated within its map keeps its far-field intensity
    (the plane wave and the far field only change phase); the training
    translations stay inside the ranges shift_ranges allows."""
    import torch
    S, gen, net, maps, inten = trained
    sub = maps[:8]
    ranges = S.shift_ranges(sub)
    moved = S.shifted(torch.tensor(sub, device="cuda"), np.arange(8), ranges, np.random.default_rng(3)).cpu().numpy()
    assert np.array_equal(moved.sum(axis=(1, 2)), sub.sum(axis=(1, 2)))   # nothing wrapped or lost
    fm = gen.far_field(moved)
    assert np.median(S.rel_err(fm, inten[:8])) < 0.02


def test_multi_view_prediction_averages_symmetric_views(trained):
    """predict(views=2) is the mean of the direct prediction and the mirrored
    structure's prediction mapped back (phi -> -phi)."""
    S, gen, net, maps, inten = trained
    sub = maps[192:200]
    direct = S.predict(net, sub)
    mirrored = S.predict(net, sub[:, :, ::-1].copy())[:, :, (360 - np.arange(360)) % 360]
    np.testing.assert_allclose(S.predict(net, sub, views=2), 0.5 * (direct + mirrored), rtol=1e-5, atol=1e-7)
    four = S.predict(net, sub, views=4)
    assert four.shape == direct.shape and np.isfinite(four).all()


def test_screening_fallback_and_audit(trained):
    S, gen, net, maps, inten = trained
    part = maps[192:256]
    # a tolerance no audit can meet: every batch falls back to FDTD
    out, st = S.screen(net, part, gen, audit_frac=0.05, tol=1e-9, batch=64)
    assert st["fallback_batches"] == st["batches"] == 1
    assert np.max(S.rel_err(out, inten[192:256])) < 1e-5
    # a tolerance every audit meets: predictions kept, audited ones replaced by FDTD
    out, st = S.screen(net, part, gen, audit_frac=0.05, tol=10.0, batch=64)
    assert st["fallback_batches"] == 0 and st["audited"] == 4
    err = S.rel_err(out, inten[192:256])
    assert np.sum(err < 1e-5) >= 4
