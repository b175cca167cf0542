"""sc_exclusive_scan_i64_noalloc (scan with its tile sums in a fixed device array, no
allocation) against sc_exclusive_scan_i64 (caller workspace), through the C ABI.

Two calls in a row, the second smaller than the first, so the second runs on an array that
still holds the first call's tile sums.  Integer results: bit-exact.  The file is named to be
collected last; it also passes on its own in a fresh process (the first call on the device
does the array's set-up)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 8388608  # SC_SCAN_NOALLOC_MAX_N


@pytest.fixture(scope="module")
def lib():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from scatter_gb300 import _native as nat

    return nat.load()


def test_noalloc_scan_matches_workspace_scan_on_two_calls(lib):
    import torch

    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(2468)
    for n in (MAX_N - 12345, 70001):  # the second call reuses the array after the first
        x_host = rng.integers(-(1 << 31), 1 << 31, size=n, dtype=np.int64)
        x = torch.from_numpy(x_host).cuda()
        out_ws = torch.full((n + 1,), -1, dtype=torch.int64, device="cuda")
        out_na = torch.full((n + 1,), -2, dtype=torch.int64, device="cuda")
        work = torch.empty(lib.sc_scan_work_size(n), dtype=torch.int64, device="cuda")
        rc_ws = lib.sc_exclusive_scan_i64(n, x.data_ptr(), out_ws.data_ptr(), work.data_ptr(), stream)
        rc_na = lib.sc_exclusive_scan_i64_noalloc(n, x.data_ptr(), out_na.data_ptr(), stream)
        torch.cuda.synchronize()
        assert rc_ws == 0, lib.sc_last_error()
        assert rc_na == 0, lib.sc_last_error()
        assert torch.equal(out_na, out_ws)
        ref = np.concatenate([[0], np.cumsum(x_host)])
        np.testing.assert_array_equal(out_na.cpu().numpy(), ref)


def test_noalloc_scan_edge_sizes_and_rejection(lib):
    import torch

    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n in (0, 1, 8192, 8193):  # empty input, one value, one full tile, a ragged second tile
        # (n = 0 still passes a real buffer: null pointers are rejected as bad arguments)
        x = torch.arange(max(n, 1), dtype=torch.int64, device="cuda") * 3 - 5
        out = torch.full((n + 1,), 99, dtype=torch.int64, device="cuda")
        assert lib.sc_exclusive_scan_i64_noalloc(n, x.data_ptr(), out.data_ptr(), stream) == 0, lib.sc_last_error()
        torch.cuda.synchronize()
        ref = np.concatenate([[0], np.cumsum(x.cpu().numpy()[:n])])
        np.testing.assert_array_equal(out.cpu().numpy(), ref)
    # beyond the maximum: rejected on the host before any launch (buffers sized for it anyway)
    n = MAX_N + 1
    x = torch.zeros(n, dtype=torch.int64, device="cuda")
    out = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    assert lib.sc_exclusive_scan_i64_noalloc(n, x.data_ptr(), out.data_ptr(), stream) == 4  # SC_CAPACITY
    assert b"exceeds the maximum" in lib.sc_last_error()
    torch.cuda.synchronize()
