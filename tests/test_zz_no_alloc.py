"""gain_dot_noalloc (the dot product that allocates no device memory) against gain_dot,
through the C ABI.  The file name puts it last in collection; it also passes on its own."""
import ctypes

import numpy as np
import pytest

MAX_N = 16384 * 4096   # GAIN_DOT_NOALLOC_MAX_N


def _noalloc(L):
    f = L.gain_dot_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def test_sizes_beyond_the_scratch_are_rejected_on_the_host(built_lib):
    """Checked before any device call: the dummy pointers are never dereferenced."""
    import gainls
    L = gainls.lib()
    f = _noalloc(L)
    assert f(MAX_N + 1, 16, 16, 16, None) == gainls.ERR_INVALID_ARG
    assert b"exceeds the scratch capacity" in L.gain_last_error_string()
    assert f(-1, 16, 16, 16, None) == gainls.ERR_INVALID_ARG
    assert f(10, 16, 16, None, None) == gainls.ERR_INVALID_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("n", [0, 1, 4095, 4096, 4097, 12345, 1_000_003, MAX_N])
def test_two_calls_in_a_row_match_gain_dot(built_lib, n):
    import torch
    import gainls
    f = _noalloc(gainls.lib())
    g = torch.Generator(device="cuda").manual_seed(17 + n)
    x = torch.randn(max(n, 1), dtype=torch.float64, device="cuda", generator=g)
    y = torch.randn(max(n, 1), dtype=torch.float64, device="cuda", generator=g)
    ref = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
    out = torch.full((2,), np.nan, dtype=torch.float64, device="cuda")
    gainls.dot(n, x.data_ptr(), y.data_ptr(), ref.data_ptr())
    for k in range(2):
        assert f(n, x.data_ptr(), y.data_ptr(), out.data_ptr() + 8 * k, None) == gainls.OK
    torch.cuda.synchronize()
    r, o = ref.item(), out.cpu().numpy()
    # both are FP64 sums of the same n products in different orders
    scale = float(torch.sum(torch.abs(x[:n] * y[:n])).item()) if n else 0.0
    tol = 4.0 * max(n, 1) * 2.0 ** -53 * scale
    assert abs(o[0] - r) <= tol and abs(o[1] - r) <= tol, (o, r, tol)
    assert o[0] == o[1]   # fixed summation order: identical on repeat
    if n == 0:
        assert o[0] == 0.0 and r == 0.0
