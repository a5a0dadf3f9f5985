"""estl_execute_noalloc: the four-step FFT for callers that cannot allocate
device memory (a host whose allocator owns all device memory, latency-critical
loops where cudaMalloc would synchronise, plugin hosts that forbid device
allocation).  Its scratch lives in a fixed 2^22-element device array.

Checked through the C ABI against the FP64 oracle (oracle.fft, the FFTW plan
semantics of FFT_FFTW3.h:23-31) at the parity tolerance of
tests/test_gpu_fft.py (rel-L2 2e-6 up to 2^20, 2 log2(N) 2^-24 beyond), for
every length the entry point accepts, both directions, with one transform
more than the fixed array holds (so each call runs at least two column / row
pairs through the same array), on two calls in a row so that the second call
runs on the first call's leftover scratch.  This file is collected last
(test_zz_*) and passes both alone in a fresh process and after the other
tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCRATCH_LOG = 22  # the fixed array: 2^22 complex64


def tol(logn):
    return 2e-6 if logn <= 20 else 2 * logn * 2.0 ** -24


def rel_l2(a, b):
    a = a.astype(np.complex128)
    b = b.astype(np.complex128)
    return np.sqrt(np.sum(np.abs(a - b) ** 2, axis=-1) / np.sum(np.abs(b) ** 2, axis=-1))


@pytest.mark.parametrize("direction", [-1, +1])
@pytest.mark.parametrize("logn", list(range(14, SCRATCH_LOG + 1)))
def test_noalloc_matches_oracle(logn, direction):
    import torch

    import oracle
    from estl_gb300._lib import check, lib

    n = 1 << logn
    batch = (1 << (SCRATCH_LOG - logn)) + 1  # one transform more than the array holds
    rng = np.random.default_rng(logn * 7 + (direction > 0))
    x = (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(np.complex64)
    ref = oracle.fft(x, direction)
    xd = torch.from_numpy(x).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    import estl_gb300 as estl
    L = lib()
    free_after, reserved_after = [], []
    y = torch.empty_like(xd)
    engine_used = estl.memory_usage()[0]
    for call in range(2):
        y.fill_(float("nan"))
        torch.cuda.synchronize()
        check(L.estl_execute_noalloc(n, batch, direction, ctypes.c_void_p(xd.data_ptr()),
                                     ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(stream)))
        torch.cuda.synchronize()
        free_after.append(torch.cuda.mem_get_info()[0])
        reserved_after.append(torch.cuda.memory_reserved())
        yh = y.cpu().numpy()
        assert np.all(np.isfinite(yh)), f"call {call}: unwritten output"
        e = rel_l2(yh, ref).max()
        assert e < tol(logn), (call, e)
    # after the first call (which may load the module's device arrays) calls
    # allocate nothing: neither the driver's free memory nor torch's pool moves
    assert reserved_after[1] == reserved_after[0]
    assert free_after[1] == free_after[0]
    # and the engine's own allocator (every device allocation of the library
    # goes through its HBM budget) is not touched by either call
    assert estl.memory_usage()[0] == engine_used


def test_noalloc_rejects_sizes_beyond_the_limit():
    import torch

    from estl_gb300._lib import lib

    L = lib()
    buf = torch.zeros(2 * (1 << 23), dtype=torch.complex64, device="cuda")
    a, b = buf.data_ptr(), buf.data_ptr() + 8 * (1 << 23)
    st = L.estl_execute_noalloc(1 << 23, 1, -1, ctypes.c_void_p(a), ctypes.c_void_p(b), None)
    assert st == 2  # ESTL_UNSUPPORTED_SIZE
    assert b"2^22" in L.estl_last_error()
    st = L.estl_execute_noalloc(1 << 10, 1, -1, ctypes.c_void_p(a), ctypes.c_void_p(b), None)
    assert st == 2
    st = L.estl_execute_noalloc(1 << 16, 1, -1, ctypes.c_void_p(a), ctypes.c_void_p(a), None)
    assert st == 1  # in-place rejected
