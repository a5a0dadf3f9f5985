"""2D transforms (FFT2D<D>, FFT.h:54-84): xdim-point FFTs over the rows of a
row-major ydim x xdim array, then ydim-point FFTs over its columns.  Here one
row pass (any 1D plan) and one in-place column pass (ColKernel without the
four-step twiddle).

* emulator (CPU): every column-tile length through the host emulator, with
  bounds checks, against the FP64 oracle applied along both axes;
* GPU: the C ABI (estl_plan2d_create + estl_execute / estl_execute_host).

Tolerance: rel-L2 per 2D array 2e-6 (the 1D FP32 target; errors of the two
passes add in quadrature).
"""
import ctypes

import numpy as np
import pytest

import oracle

TOL = 2e-6


def rand_c64(shape, seed):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64)


def fft2_oracle(x, sign):
    """FP64 2D DFT of (batch, ydim, xdim) arrays: rows, then columns."""
    y = oracle.fft(x, sign)
    y = oracle.fft(np.ascontiguousarray(np.swapaxes(y, -1, -2)), sign)
    return np.swapaxes(y, -1, -2)


def rel_l2_arrays(y, ref):
    d = (y.astype(np.complex128) - ref).reshape(y.shape[0], -1)
    r = ref.reshape(ref.shape[0], -1)
    return np.sqrt(np.sum(np.abs(d) ** 2, axis=1) / np.sum(np.abs(r) ** 2, axis=1))


def emu2d(emu, x, sign):
    batch, ydim, xdim = x.shape
    y = np.full(x.shape, np.nan + 1j * np.nan, np.complex64)
    err = ctypes.create_string_buffer(512)
    rc = emu.emu_plan2d_run(xdim, ydim, batch, sign, x.ctypes.data, y.ctypes.data, err, len(err))
    return rc, err.value.decode(), y


@pytest.mark.parametrize("logy", range(0, 13))
def test_emulated_2d_every_column_length(emu, logy):
    for logx, batch in ((0, 3), (1, 2), (3, 2), (6, 2), (10, 1)):
        if logx + logy > 16:
            continue
        x = rand_c64((batch, 1 << logy, 1 << logx), 10 * logy + logx)
        for sign in (-1, +1):
            rc, msg, y = emu2d(emu, x, sign)
            assert rc == 0, (logx, logy, msg)
            assert rel_l2_arrays(y, fft2_oracle(x, sign)).max() < TOL, (logx, logy, sign)


def test_emulated_2d_four_step_rows(emu):
    """Rows longer than 2^14 run the four-step row plan before the column pass."""
    x = rand_c64((1, 4, 1 << 15), 5)
    rc, msg, y = emu2d(emu, x, -1)
    assert rc == 0, msg
    assert rel_l2_arrays(y, fft2_oracle(x, -1)).max() < TOL


def test_emulated_2d_rejects(emu):
    x = rand_c64((1, 1 << 13, 2), 1)
    rc, msg, _ = emu2d(emu, x, -1)
    assert rc == 2 and "ydim" in msg
    x = rand_c64((1, 3, 4), 1)
    rc, msg, _ = emu2d(emu, x, -1)
    assert rc == 2 and "powers of two" in msg


@pytest.mark.gpu
@pytest.mark.parametrize("xdim,ydim,batch", [(1, 64, 3), (16, 16, 7), (4096, 4096, 1), (2048, 512, 3),
                                             (1 << 16, 64, 2), (256, 4096, 2), (8, 1024, 5), (1 << 20, 8, 1)])
def test_gpu_2d_parity(engine, xdim, ydim, batch):
    import torch
    x = rand_c64((batch, ydim, xdim), xdim + ydim + batch)
    xd = torch.from_numpy(x).cuda()
    for sign in (-1, +1):
        p = engine.Plan2D(xdim, ydim, batch, sign)
        d = p.describe()
        assert d["xdim"] == xdim and d["ydim"] == ydim
        if ydim > 1:
            assert d["kernels"][-1]["kind"] == "column"
        y = p.execute(xd).cpu().numpy()
        assert rel_l2_arrays(y, fft2_oracle(x, sign)).max() < TOL, (xdim, ydim, sign)


@pytest.mark.gpu
def test_gpu_2d_round_trip_and_host(engine):
    """backward(forward(x)) / (xdim * ydim) = x; estl_execute_host is bit-identical
    to estl_execute."""
    import torch
    xdim, ydim, batch = 1024, 256, 6
    x = rand_c64((batch, ydim, xdim), 77)
    xd = torch.from_numpy(x).cuda()
    f = engine.Plan2D(xdim, ydim, batch, -1)
    b = engine.Plan2D(xdim, ydim, batch, +1)
    y = f.execute(xd)
    z = b.execute(y).cpu().numpy() / (xdim * ydim)
    assert rel_l2_arrays(z, x.astype(np.complex128)).max() < TOL
    h = np.empty_like(x)
    f.execute_host(x, h)
    assert np.array_equal(h, y.cpu().numpy())
