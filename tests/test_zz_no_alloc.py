"""estl_execute_noalloc: the four-step FFT for callers that cannot allocate
device memory (a host whose allocator owns all device memory, latency-critical
loops where cudaMalloc would synchronise, plugin hosts that forbid device
allocation).  Its scratch lives in a fixed 2^22-element device array.

Checked through the C ABI against the plan-based entry point (estl_execute),
within the parity tolerance of tests/test_gpu_fft.py (rel-L2 2e-6), on two
calls in a row so that the second call runs on the first call's leftover
scratch.  This file is collected last (test_zz_*) and passes both alone in a
fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-6


def rel_l2(a, b):
    a = a.astype(np.complex128)
    b = b.astype(np.complex128)
    return np.sqrt(np.sum(np.abs(a - b) ** 2, axis=-1) / np.sum(np.abs(b) ** 2, axis=-1))


@pytest.mark.parametrize("logn,batch,direction", [(14, 9, -1), (16, 5, -1), (20, 3, +1), (22, 2, -1)])
def test_noalloc_matches_plan_execute(logn, batch, direction):
    import torch

    import estl_gb300 as estl
    from estl_gb300._lib import check, lib

    n = 1 << logn
    rng = np.random.default_rng(logn * 7 + batch)
    x = (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    ref = estl.Plan(n, batch, direction).execute(xd)
    torch.cuda.synchronize()
    ref_h = ref.cpu().numpy()
    stream = torch.cuda.current_stream().cuda_stream
    L = lib()
    free_after = []
    y = torch.empty_like(xd)
    for call in range(2):
        y.fill_(float("nan"))
        torch.cuda.synchronize()
        check(L.estl_execute_noalloc(n, batch, direction, ctypes.c_void_p(xd.data_ptr()),
                                     ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(stream)))
        torch.cuda.synchronize()
        free_after.append(torch.cuda.mem_get_info()[0])
        yh = y.cpu().numpy()
        assert np.all(np.isfinite(yh)), f"call {call}: unwritten output"
        e = rel_l2(yh, ref_h).max()
        assert e < TOL, (call, e)
    # after the first call (which may load the module's device arrays), calls allocate nothing
    assert free_after[1] == free_after[0]


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
