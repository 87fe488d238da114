"""The surrogate's hand-written forward/backward kernels against the CPU
oracle (oracle/surrogate_ref.py), and a short training run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_surrogate_gradients_match_cpu_oracle():
    import torch
    from mpifdtd_gb300.surrogate import model as Mdl
    from oracle import surrogate_ref as R
    rng = np.random.default_rng(3)
    B = 128
    maps = (rng.random((B, 256, 256)) < 0.15).astype(np.uint8)
    y = rng.normal(0, 1, (B, Mdl.NT)).astype(np.float32)
    params = Mdl.init_params(7)
    net = Mdl.FNO(params)
    x = net.pool(torch.tensor(maps, device="cuda"))
    w = rng.uniform(0.5, 2.0, B).astype(np.float32)   # per-structure loss weights
    loss, g = net.loss_and_grads(x, torch.tensor(y, device="cuda"), torch.tensor(w, device="cuda"))
    torch.cuda.synchronize()
    from mpifdtd_gb300.surrogate import kernels as K
    assert int(K.err_word().item()) == 0
    x_cpu = R.pool_map(maps)
    np.testing.assert_allclose(x.cpu().numpy(), x_cpu, rtol=0, atol=1e-7)
    D, E = Mdl.basis()
    loss_ref, g_ref = R.loss_and_grads(params, x_cpu, y.astype(np.float64), D, E, w.astype(np.float64))
    assert _rel(loss.cpu().numpy(), loss_ref) < 1e-3
    for k, ref in g_ref.items():
        e = _rel(g[k].cpu().numpy().astype(np.float64), ref)
        assert e < 2e-2, (k, e)


def test_surrogate_training_reduces_loss_on_fixed_batch():
    import torch
    from mpifdtd_gb300.surrogate import model as Mdl
    rng = np.random.default_rng(4)
    B = 128
    maps = torch.tensor((rng.random((B, 256, 256)) < 0.2).astype(np.uint8), device="cuda")
    net = Mdl.FNO(seed=5)
    x = net.pool(maps)
    # targets: a smooth function of the map the network can represent
    y = torch.tensor(rng.normal(0, 0.1, (B, Mdl.NT)), device="cuda", dtype=torch.float32)
    y += x[0].mean(1, keepdim=True) * 5.0
    first = None
    for it in range(60):
        loss, g = net.loss_and_grads(x, y)
        net.adam_step(g, lr=1e-3)
        if first is None:
            first = float(loss.mean())
    last = float(loss.mean())
    assert last < 0.25 * first, (first, last)
