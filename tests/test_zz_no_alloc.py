"""gain_dot_noalloc, the dot product for callers that cannot allocate device memory (a host
program whose device memory is all handed out by its own pool allocator, so that a direct
cudaMalloc would fail or break its budget), checked through the C ABI against a host FP64 sum
of the same products and against gain_dot.  The file name puts it last in collection; it
also passes on its own in a fresh process."""
import ctypes
import math

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
def test_two_calls_in_a_row_match_host_sum(built_lib, n):
    import torch
    import gainls
    f = _noalloc(gainls.lib())
    rng = np.random.default_rng(17 + n)
    xh = rng.standard_normal(max(n, 1))
    yh = rng.standard_normal(max(n, 1))
    x = torch.from_numpy(xh).cuda()
    y = torch.from_numpy(yh).cuda()
    ref = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
    out = torch.full((2,), np.nan, dtype=torch.float64, device="cuda")
    gainls.dot(n, x.data_ptr(), y.data_ptr(), ref.data_ptr())
    for k in range(2):
        assert f(n, x.data_ptr(), y.data_ptr(), out.data_ptr() + 8 * k, None) == gainls.OK
    torch.cuda.synchronize()
    o, r_dev = out.cpu().numpy(), ref.item()
    # host reference: the correctly rounded sum of the FP64 products (math.fsum)
    prod = xh[:n] * yh[:n]
    host = math.fsum(prod) if n else 0.0
    # the device sums the exact products (fused multiply-adds) in a fixed order: its error
    # and the products' own roundings are each within n 2^-53 sum |x y|
    scale = float(np.sum(np.abs(prod))) if n else 0.0
    tol = 4.0 * max(n, 1) * 2.0 ** -53 * scale
    assert abs(o[0] - host) <= tol and abs(o[1] - host) <= tol, (o, host, tol)
    assert abs(r_dev - host) <= tol   # the allocating entry point agrees as well
    assert o[0] == o[1]   # fixed summation order: identical on repeat
    if n == 0:
        assert o[0] == 0.0 and host == 0.0
