"""GPU test of ngb_dot_noalloc, the dot product for callers that cannot
allocate device memory. It is called through the C ABI and must agree with
ngb_dot (caller scratch) on the same inputs, on two calls in a row (the second
call reuses the library's fixed scratch left over from the first), within the
FP64-summation-order tolerance of the other dot tests. This file is collected
last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib(ngb):
    L = ngb.lib()
    L.ngb_dot_noalloc.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p]
    L.ngb_dot_noalloc.restype = ctypes.c_int
    return L


def _noalloc(L, ngb, a, b, out):
    import torch
    field = ngb.STORE_F64 if a.dtype == torch.float64 else ngb.STORE_F32
    return L.ngb_dot_noalloc(a.numel(), field, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                             ctypes.c_void_p(out.data_ptr()), None)


@pytest.mark.parametrize("dtype,n", [("float32", 3_000_001), ("float64", 1_048_576), ("float32", 8191)])
def test_dot_noalloc_matches_dot_twice(ngb, cuda, dtype, n):
    import torch
    L = _lib(ngb)
    dt = getattr(torch, dtype)
    g = torch.Generator().manual_seed(1234 + n)
    for call in range(2):  # two calls in a row on different data
        a = torch.randn(n, generator=g, dtype=torch.float64).to(dt).to(cuda)
        b = torch.randn(n, generator=g, dtype=torch.float64).to(dt).to(cuda)
        ref = torch.zeros(1, dtype=torch.float64, device=cuda)
        got = torch.full((1,), float("nan"), dtype=torch.float64, device=cuda)
        ngb.dot(a, b, ref)
        assert _noalloc(L, ngb, a, b, got) == 0, L.ngb_last_error()
        torch.cuda.synchronize()
        r, x = ref.item(), got.item()
        assert abs(x - r) <= 1e-12 * max(1.0, np.sqrt(n)), (call, x, r)


def test_dot_noalloc_rejects_oversize(ngb, cuda):
    import torch
    L = _lib(ngb)
    a = torch.zeros(4, device=cuda)
    out = torch.zeros(1, dtype=torch.float64, device=cuda)
    rc = L.ngb_dot_noalloc((1 << 28) + 1, ngb.STORE_F32, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(a.data_ptr()),
                           ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -4
    assert b"exceeds the maximum" in L.ngb_last_error()
