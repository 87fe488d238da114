"""ctypes bindings of libmpifdtd_surrogate.so over torch tensors.

torch provides device memory and the current stream; every computation runs
in the library's own kernels (tcgen05 GEMM, element-wise kernels, Adam)."""
from __future__ import annotations

import ctypes as C

from .. import build as _build

_lib = None
P, I, F = C.c_void_p, C.c_int, C.c_float


class SurrogateError(RuntimeError):
    pass


def load():
    global _lib
    if _lib is not None:
        return _lib
    so = _build.SURROGATE_SO
    if not so.exists():
        raise ImportError(f"surrogate library missing ({so}); run mpifdtd_gb300.build.build()")
    lib = C.CDLL(str(so))
    L = C.c_longlong
    lib.sg_gemm_bf16_tn.restype = I
    lib.sg_gemm_bf16_tn.argtypes = [P, I, P, I, P, I, I, I, I, I, I, P, I, P, P, P]
    lib.sg_gemm_bf16_tn_batched.restype = I
    lib.sg_gemm_bf16_tn_batched.argtypes = [P, I, L, P, I, L, P, I, L, I, I, I, I, I, I, P, I, P, P, P]
    lib.sg_last_error.restype = C.c_char_p
    for name, args in _OPS.items():
        f = getattr(lib, name)
        f.restype = I
        f.argtypes = args
    _lib = lib
    return lib


L_ = C.c_longlong
_OPS: dict = {
    "sg_pool_map": [P, P, I, P],
    "sg_lift": [P, P, P, P, P, I, I, P],
    "sg_lift_bwd": [P, P, P, P, I, I, P],
    "sg_mode_permute": [P, P, I, I, I, I, P],
    "sg_act_fwd": [P, P, P, I, I, I, P],
    "sg_act_bwd": [P, P, P, P, P, I, I, I, P],
    "sg_colsum_f32": [P, P, I, I, P],
    "sg_head_pool": [P, P, I, I, I, P],
    "sg_head_unpool": [P, P, I, I, I, P],
    "sg_amp_mse": [P, P, P, P, P, I, I, I, P],
    "sg_gelu_bwd": [P, P, P, L_, P],
    "sg_colsum": [P, P, I, I, P],
    "sg_transpose": [P, P, I, I, I, P],
    "sg_cast_bf16": [P, P, L_, P],
    "sg_adam": [P, P, P, P, P, L_, F, F, F, F, F, F, F, P],
}


def op(name, *args):
    """Launch one element-wise kernel of the library on the current stream."""
    conv = [_ptr(a) if hasattr(a, "data_ptr") else a for a in args]
    rc = getattr(load(), name)(*conv, _stream())
    if rc != 0:
        raise SurrogateError(f"{name} failed ({rc})")


def transpose(a, out=None):
    """[Z,]R,C bf16 -> [Z,]C,R (contiguous)."""
    import torch
    z, r, c = (a.shape if a.dim() == 3 else (1,) + tuple(a.shape))
    if out is None:
        out = torch.empty((z, c, r) if a.dim() == 3 else (c, r), dtype=a.dtype, device=a.device)
    assert a.is_contiguous() and out.is_contiguous()
    op("sg_transpose", a, out, z, r, c)
    return out


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check(rc):
    if rc != 0:
        raise SurrogateError(load().sg_last_error().decode())


_err = None


def err_word():
    """Device status word of the GEMM's bounded waits (0 = no timeout)."""
    import torch
    global _err
    if _err is None:
        _err = torch.zeros(1, dtype=torch.int32, device="cuda")
    return _err


def gemm(a, b, out, bias=None, act=0, accumulate=False, pre=None):
    """out[M,N] = a[M,K] . b[N,K]^T (+bias) (+out) (GELU if act=1); a, b BF16
    row-major (last dim contiguous, leading dims may be strided views of
    rows), out FP32 or BF16; pre: FP32 [M,N] copy of the pre-activation.
    Batched when out is 3-D: out[Z,M,N] with a[Z,M,K] or a shared a[M,K], and
    b[Z,N,K] or a shared b[N,K] (at least one of a, b per batch entry)."""
    import torch
    assert a.dtype == torch.bfloat16 and b.dtype == torch.bfloat16
    assert a.stride(-1) == 1 and b.stride(-1) == 1 and out.stride(-1) == 1
    z = out.shape[0] if out.dim() == 3 else 1
    m, k = a.shape[-2:]
    n, k2 = b.shape[-2:]
    assert k == k2 and tuple(out.shape[-2:]) == (m, n)
    abs_ = a.stride(0) if a.dim() == 3 else 0
    bbs = b.stride(0) if b.dim() == 3 else 0
    cbs = out.stride(0) if out.dim() == 3 else 0
    if pre is not None:
        assert pre.stride() == out.stride()
    c_bf16 = 1 if out.dtype == torch.bfloat16 else 0
    _check(load().sg_gemm_bf16_tn_batched(_ptr(a), a.stride(-2), abs_, _ptr(b), b.stride(-2), bbs, _ptr(out),
                                          out.stride(-2), cbs, m, n, k, z, c_bf16, 1 if accumulate else 0,
                                          _ptr(bias), act, _ptr(pre), _ptr(err_word()), _stream()))
    return out
