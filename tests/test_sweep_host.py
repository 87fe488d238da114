"""Host-side logic of the batched sweep workload and of the surrogate's training translations (no GPU)."""
import numpy as np


def test_sweep_cases_follow_the_workload_definition():
    from mpifdtd_gb300.sweep import mie_sweep
    cases = mie_sweep(256)
    assert len(cases) == 256
    for c in cases:
        n = c.fi.width_nm // 5
        assert n == int(np.ceil((2 * c.radius_nm + 2 * c.lambda_nm) / 5)) + 20
        assert 100 <= c.radius_nm <= 800 and 1.5 <= c.eps <= 4.0 and 380 <= c.lambda_nm <= 780
        assert c.fi.step_num == int(np.ceil(12 * (c.lambda_nm / 5) / 0.7071))


def test_surrogate_shift_ranges_keep_structures_inside():
    """The translations drawn for training keep every structure at least 6
    cells inside its 256^2 map, or do not move it towards an edge it is
    already nearer than that."""
    from mpifdtd_gb300.surrogate.data import make_maps
    from mpifdtd_gb300.surrogate.screen import shift_ranges
    maps = make_maps(64, 11)
    r = shift_ranges(maps)
    assert (r[:, 0] <= 0).all() and (r[:, 1] >= 0).all() and (r[:, 2] <= 0).all() and (r[:, 3] >= 0).all()
    for m, (x0, x1, y0, y1) in zip(maps, r):
        xs = np.nonzero(m.any(axis=1))[0]
        ys = np.nonzero(m.any(axis=0))[0]
        for lo, hi, a, b in ((xs[0], xs[-1], x0, x1), (ys[0], ys[-1], y0, y1)):
            assert lo + a >= min(lo, 6) and hi + b <= max(hi, 249)
