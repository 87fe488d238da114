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
    lib.sg_gemm_bf16_tn.restype = I
    lib.sg_gemm_bf16_tn.argtypes = [P, I, P, I, P, I, I, I, I, I, I, P, I, P, P, P]
    lib.sg_last_error.restype = C.c_char_p
    for name, args in _OPS.items():
        f = getattr(lib, name)
        f.restype = I
        f.argtypes = args
    _lib = lib
    return lib


_OPS: dict = {}


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
    rows), out FP32 or BF16; pre: FP32 [M,N] copy of the pre-activation."""
    import torch
    assert a.dtype == torch.bfloat16 and b.dtype == torch.bfloat16
    assert a.stride(1) == 1 and b.stride(1) == 1 and out.stride(1) == 1
    m, k = a.shape
    n, k2 = b.shape
    assert k == k2 and out.shape == (m, n)
    c_bf16 = 1 if out.dtype == torch.bfloat16 else 0
    _check(load().sg_gemm_bf16_tn(_ptr(a), a.stride(0), _ptr(b), b.stride(0), _ptr(out), out.stride(0), m, n, k,
                                  c_bf16, 1 if accumulate else 0, _ptr(bias), act, _ptr(pre),
                                  _ptr(err_word()), _stream()))
    return out
