"""Lengths that are not powers of two (f4): Bluestein's algorithm over the
power-of-two plans (bluestein_core.cuh).  The reference rounds every length
up to a power of two (SimpleMath.h:7-11, FFT_OpenCL_Contiguous.h:56) and so
computes a different transform for these lengths; the target is the DFT of
the given length, as FFTW computes it (FFT_FFTW3.h:26-28).

* emulator (CPU): the same element functions around emulated FFT plans,
  against the oracle's long-double direct DFT;
* GPU: estl_plan_create with such lengths, against the direct DFT for
  moderate n and numpy's FP64 pocketfft (any length) for large n.

Tolerance: rel-L2 2e-6, the FP32 target of the power-of-two path.
"""
import ctypes

import numpy as np
import pytest

import oracle

TOL = 2e-6


def rand_c64(shape, seed):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64)


def direct(x, sign):
    return np.stack([oracle.dft_ld(row, sign) for row in x])


def rel(y, ref):
    y = y.astype(np.complex128)
    return np.sqrt(np.sum(np.abs(y - ref) ** 2, axis=-1) / np.sum(np.abs(ref) ** 2, axis=-1))


def emu_blue(emu, x, sign):
    batch, n = x.shape
    y = np.full(x.shape, np.nan + 1j * np.nan, np.complex64)
    err = ctypes.create_string_buffer(512)
    rc = emu.emu_bluestein_run(n, batch, sign, x.ctypes.data, y.ctypes.data, err, len(err))
    return rc, err.value.decode(), y


@pytest.mark.parametrize("n", [3, 5, 12, 100, 1000])
def test_emulated_bluestein_golden(emu, n):
    """The Bluestein kernels (emulated) against the mpmath golden vectors."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "dft_golden.npz"))
    for sign in (-1, +1):
        x, ref = g[f"x_{n}_{sign}"], g[f"y_{n}_{sign}"]
        rc, msg, y = emu_blue(emu, np.ascontiguousarray(x[None, :]), sign)
        assert rc == 0, msg
        assert rel(y, ref[None, :]).max() < TOL, (n, sign)


@pytest.mark.parametrize("n", [3, 5, 6, 7, 12, 15, 100, 243, 1000, 3000])
def test_emulated_bluestein(emu, n):
    x = rand_c64((3, n), n)
    for sign in (-1, +1):
        rc, msg, y = emu_blue(emu, x, sign)
        assert rc == 0, msg
        assert rel(y, direct(x, sign)).max() < TOL, (n, sign)


@pytest.mark.parametrize("n", [8191, 8193, 9000, 40000])
def test_emulated_bluestein_four_step(emu, n):
    """Both sides of the fused / four-step boundary (8191: M = 2^14, the last
    fused length; 8193: M = 2^15), and M = 2^15 and 2^17: the three four-step
    kernels with the chirps folded into the first load and the last store
    (emulated, bounds-checked), against the oracle's direct DFT on sampled
    bins."""
    x = rand_c64((2, n), n)
    rng = np.random.default_rng(n)
    bins = np.concatenate([[0, 1, n // 2, n - 1], rng.integers(0, n, 28)])
    for sign in (-1, +1):
        rc, msg, y = emu_blue(emu, x, sign)
        assert rc == 0, msg
        for b in range(2):
            ref = oracle.dft_bins(x[b], bins, sign)
            e = np.sqrt(np.sum(np.abs(y[b, bins] - ref) ** 2) / np.sum(np.abs(ref) ** 2))
            assert e < TOL, (n, sign, b, e)


def test_emulated_bluestein_rejects(emu):
    for n in (1, 2, 16, (1 << 23) + 1):
        x = np.zeros((1, 4), np.complex64)
        err = ctypes.create_string_buffer(512)
        rc = emu.emu_bluestein_run(n, 1, -1, x.ctypes.data, x.ctypes.data, err, len(err))
        assert rc == 2, n


@pytest.mark.gpu
@pytest.mark.parametrize("n,batch", [(3, 7), (12, 5), (1000, 9), (4095, 3), (8191, 3), (8193, 3), (10000, 2),
                                     (123457, 2), (1000000, 2), ((1 << 21) - 1, 1), ((1 << 21) + 1, 1),
                                     ((1 << 23) - 1, 1)])
def test_gpu_bluestein(engine, n, batch):
    import torch
    x = rand_c64((batch, n), n % 1000 + batch)
    xd = torch.from_numpy(x).cuda()
    for sign in (-1, +1):
        p = engine.Plan(n, batch, sign)
        d = p.describe()
        assert d["bluestein_m"] >= 2 * n - 1
        y = p.execute(xd).cpu().numpy()
        if n <= 4096:
            ref = direct(x, sign)
            assert rel(y, ref).max() < TOL, (n, sign)
        else:
            # the oracle's direct DFT (no FFT involved) on 24 sampled bins per
            # transform (both ends and random ones), relative to the bins' norm
            rng = np.random.default_rng(n)
            bins = np.concatenate([[0, 1, n // 2, n - 1], rng.integers(0, n, 20)])
            for b in range(batch):
                ref_b = oracle.dft_bins(x[b], bins, sign)
                e = np.sqrt(np.sum(np.abs(y[b, bins] - ref_b) ** 2) / np.sum(np.abs(ref_b) ** 2))
                assert e < TOL, (n, sign, b, e)


@pytest.mark.gpu
def test_gpu_bluestein_host_and_many_chunks(engine):
    """A batch larger than one pass through the M-point FFTs (several chunks),
    and estl_execute_host bit-identical to estl_execute."""
    import torch
    n, batch = 3 << 17, 150  # M = 2^20: chunks of 64 transforms (64 + 64 + 22)
    x = rand_c64((batch, n), 3)
    p = engine.Plan(n, batch, -1)
    assert p.describe()["bluestein_m"] == 1 << 20
    y = p.execute(torch.from_numpy(x).cuda()).cpu().numpy()
    ref = np.fft.fft(x[::37].astype(np.complex128), axis=-1)
    assert rel(y[::37], ref).max() < TOL
    h = np.empty_like(x)
    p.execute_host(x, h)
    assert np.array_equal(h, y)
