"""tcgen05 BF16 GEMM of the surrogate against an FP32 product of the same
BF16 operands (FP32 accumulation: agreement to FP32 summation-order noise)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (256, 192, 128), (384, 128, 512), (128, 64, 1024),
                                   (512, 256, 320)])
def test_gemm_bf16_matches_fp32_product(m, n, k):
    import torch
    from mpifdtd_gb300.surrogate import kernels as K
    g = torch.Generator(device="cuda").manual_seed(m * 7 + n * 3 + k)
    a = torch.randn(m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16)
    ref = a.float() @ b.float().t()
    out = torch.empty(m, n, device="cuda", dtype=torch.float32)
    K.gemm(a, b, out)
    torch.cuda.synchronize()
    assert int(K.err_word().item()) == 0
    rel = (out - ref).norm() / ref.norm()
    assert rel < 1e-5, float(rel)


def test_gemm_epilogue_bias_gelu_accumulate_bf16():
    import torch
    from mpifdtd_gb300.surrogate import kernels as K
    g = torch.Generator(device="cuda").manual_seed(5)
    m, n, k = 256, 128, 192
    a = torch.randn(m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(n, device="cuda", generator=g)
    pre_ref = a.float() @ b.float().t() + bias
    gelu_ref = torch.nn.functional.gelu(pre_ref, approximate="tanh")
    out = torch.empty(m, n, device="cuda", dtype=torch.bfloat16)
    pre = torch.empty(m, n, device="cuda", dtype=torch.float32)
    K.gemm(a, b, out, bias=bias, act=1, pre=pre)
    acc = torch.ones(m, n, device="cuda", dtype=torch.float32)
    K.gemm(a, b, acc, accumulate=True)
    torch.cuda.synchronize()
    assert int(K.err_word().item()) == 0
    assert float((pre - pre_ref).norm() / pre_ref.norm()) < 1e-5
    assert float((out.float() - gelu_ref).norm() / gelu_ref.norm()) < 1e-2   # BF16 output rounding
    base = a.float() @ b.float().t() + 1.0
    assert float((acc - base).norm() / base.norm()) < 1e-5


def test_gemm_strided_operand_views():
    """Row-strided views (the model's DFT stages slice wider buffers)."""
    import torch
    from mpifdtd_gb300.surrogate import kernels as K
    g = torch.Generator(device="cuda").manual_seed(9)
    big = torch.randn(256, 320, device="cuda", generator=g).to(torch.bfloat16)
    a = big[:, 64:256]          # K = 192, lda = 320
    b = torch.randn(128, 192, device="cuda", generator=g).to(torch.bfloat16)
    out = torch.zeros(256, 256, device="cuda")[:, :128]
    K.gemm(a, b, out)
    torch.cuda.synchronize()
    ref = a.float() @ b.float().t()
    assert float((out - ref).norm() / ref.norm()) < 1e-5


@pytest.mark.parametrize("shared_b", [False, True])
def test_gemm_batched(shared_b):
    """grid.z products (3-D tensor maps), B per entry or shared."""
    import torch
    from mpifdtd_gb300.surrogate import kernels as K
    g = torch.Generator(device="cuda").manual_seed(11)
    z, m, n, k = 37, 128, 128, 128
    a = torch.randn(z, m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16) if shared_b else \
        torch.randn(z, n, k, device="cuda", generator=g).to(torch.bfloat16)
    out = torch.empty(z, m, n, device="cuda", dtype=torch.bfloat16)
    K.gemm(a, b, out)
    torch.cuda.synchronize()
    assert int(K.err_word().item()) == 0
    bt = b.float().t() if shared_b else b.float().transpose(1, 2)
    ref = a.float() @ bt
    assert float((out.float() - ref).norm() / ref.norm()) < 1e-2


def test_gemm_batched_shared_a():
    """A shared by every batch entry, B per entry (the inverse DFT into the
    channels-last layout: out[z] = E . Yt[z]^T)."""
    import torch
    from mpifdtd_gb300.surrogate import kernels as K
    g = torch.Generator(device="cuda").manual_seed(13)
    z, m, n, k = 19, 1024, 64, 512
    a = torch.randn(m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(z, n, k, device="cuda", generator=g).to(torch.bfloat16)
    out = torch.empty(z, m, n, device="cuda", dtype=torch.float32)
    K.gemm(a, b, out)
    torch.cuda.synchronize()
    assert int(K.err_word().item()) == 0
    ref = a.float() @ b.float().transpose(1, 2)
    assert float((out - ref).norm() / ref.norm()) < 1e-5


@pytest.mark.parametrize("m", [64, 192])
def test_gemm_rows_not_a_multiple_of_the_tile(m):
    """M = 64 (and 192): the last row tile reads zeros past M through the
    tensor map's fill and stores only rows below M; the rows after the output
    (a sentinel) stay untouched.  Batched, as the point-wise mixing's weight
    gradient uses it."""
    import torch
    from mpifdtd_gb300.surrogate import kernels as K
    g = torch.Generator(device="cuda").manual_seed(m)
    z, n, k = 5, 64, 1024
    a = torch.randn(z, m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(z, n, k, device="cuda", generator=g).to(torch.bfloat16)
    big = torch.full((z + 1, m, n), 7.0, device="cuda", dtype=torch.float32)
    out = big[:z]
    K.gemm(a, b, out)
    torch.cuda.synchronize()
    assert int(K.err_word().item()) == 0
    ref = a.float() @ b.float().transpose(1, 2)
    assert float((out - ref).norm() / ref.norm()) < 1e-5
    assert bool((big[z] == 7.0).all())
