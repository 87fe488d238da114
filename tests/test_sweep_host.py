"""Host-side definition of the batched sweep workload (no GPU)."""
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
