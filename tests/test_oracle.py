"""Pins the FP64 oracle before the other tests trust its results.

* the known-answer test of the reference (tests/Test.cpp:60-77): a cosine of
  frequency effK transforms to M/2 at q = effK and q = M - effK, 0 elsewhere,
  checked with the reference's own tolerance |d|^2 < 1e-3 * M and with a tight
  FP64 bound;
* golden vectors computed with mpmath (tests/golden/make_golden.py);
* a long-double direct DFT and numpy.fft (pocketfft);
* the FP32 restatement of the reference's contiguous Stockham algorithm.
"""
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "dft_golden.npz")


def reference_known_answer(M, k, batch):
    """Inputs and expected outputs of TestFourierFloat::execute for one k."""
    x = np.empty((batch, M), dtype=np.complex128)
    y = np.zeros((batch, M), dtype=np.complex128)
    q = np.arange(M)
    for b in range(batch):
        eff = ((k + b) % (M // 2 - 1)) + 1
        x[b] = np.cos(2 * np.pi * ((1.0 * eff * q) / M)).astype(np.float32)
        y[b, eff] += M / 2.0
        y[b, M - eff] += M / 2.0
    return x, y


@pytest.mark.parametrize("m", range(2, 13))
def test_known_answer_cosine(m):
    M = 1 << m
    batch = 4
    for k in range(1, min(M // 2, 6)):
        x, expect = reference_known_answer(M, k, batch)
        y = oracle.fft(x, -1)
        d2 = np.abs(y - expect) ** 2
        assert d2.max() < 1e-3 * M  # tests/Test.cpp:75 (MAX_ERR * M)
        # the input cosine is rounded to FP32 (as in the reference), which
        # moves the ideal spectrum by at most ~sqrt(M) * 2^-24 per bin
        assert np.abs(y - expect).max() < 1e-7 * M


def test_golden_vectors():
    g = np.load(GOLDEN)
    for logn in range(0, 9):
        n = 1 << logn
        for sign in (-1, +1):
            x, y = g[f"x_{n}_{sign}"], g[f"y_{n}_{sign}"]
            out = oracle.fft(x[None, :], sign)[0]
            assert oracle.rel_l2(out, y) < 1e-14, (n, sign)
    out = oracle.fft(g["kat_x"][None, :], -1)[0]
    assert np.abs(out - g["kat_y"]).max() < 1e-12


@pytest.mark.parametrize("n", [3, 5, 12, 100, 1000])
def test_golden_vectors_other_lengths(n):
    """The long-double direct DFT, the target of the lengths that are not
    powers of two, against the mpmath golden vectors of those lengths."""
    g = np.load(GOLDEN)
    for sign in (-1, +1):
        x, y = g[f"x_{n}_{sign}"], g[f"y_{n}_{sign}"]
        assert oracle.rel_l2(oracle.dft_ld(x.astype(np.complex128), sign), y) < 1e-15, (n, sign)


@pytest.mark.parametrize("logn", [1, 2, 3, 5, 8, 10])
def test_against_long_double_dft(logn):
    n = 1 << logn
    rng = np.random.default_rng(logn)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for sign in (-1, +1):
        ref = oracle.dft_ld(x, sign)
        out = oracle.fft(x[None, :], sign)[0]
        assert oracle.rel_l2(out, ref) < 1e-14


@pytest.mark.parametrize("logn", [0, 4, 11, 16, 20])
def test_against_numpy(logn):
    n = 1 << logn
    batch = max(1, min(8, (1 << 20) // n))
    rng = np.random.default_rng(100 + logn)
    x = rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))
    assert oracle.rel_l2(oracle.fft(x, -1), np.fft.fft(x, axis=-1)).max() < 1e-13
    assert oracle.rel_l2(oracle.fft(x, +1), np.fft.ifft(x, axis=-1) * n).max() < 1e-13


def test_round_trip_and_threads():
    rng = np.random.default_rng(7)
    x = rng.standard_normal((33, 1024)) + 1j * rng.standard_normal((33, 1024))
    y1 = oracle.fft(x, -1, nthreads=1)
    y8 = oracle.fft(x, -1, nthreads=8)
    assert np.array_equal(y1, y8)
    z = oracle.fft(y8, +1) / 1024
    assert oracle.rel_l2(z, x).max() < 1e-15


def test_rejects_non_power_of_two():
    with pytest.raises(ValueError):
        oracle.fft(np.zeros((1, 12), np.complex128))


@pytest.mark.parametrize("la,lb", [(1, 1), (5, 3), (100, 17), (256, 16), (1000, 64)])
def test_conv_fft_matches_direct(la, lb):
    rng = np.random.default_rng(la * 31 + lb)
    a, b = rng.standard_normal(la), rng.standard_normal(lb)
    direct = oracle.conv_direct(a, b)
    assert np.allclose(oracle.conv_fft(a, b), direct, rtol=0, atol=1e-12 * np.abs(direct).max())
    assert np.allclose(direct, np.convolve(a, b), rtol=0, atol=1e-12 * np.abs(direct).max())
    corr = oracle.conv_fft(a, b, correlate=True)
    # correlation is convolution with the reversed filter, circularly shifted by lb-1 in a length-n buffer
    n = 1 << int(np.ceil(np.log2(la + lb - 1))) if la + lb - 1 > 1 else 1
    full = np.zeros(n)
    for m in range(n):
        full[m] = sum(a[i] * b[(i - m) % n] if 0 <= (i - m) % n < lb else 0.0 for i in range(la))
    assert np.allclose(corr, full[: la + lb - 1], atol=1e-9 * max(1, np.abs(full).max()))


@pytest.mark.parametrize("logn", [1, 4, 6, 12, 13, 16])
def test_reference_algorithm_port(logn):
    """The FP32 restatement of FFT_OpenCL_Contiguous agrees with the oracle to
    the accuracy its 6-digit twiddles allow (2*pi streamed as 6.28319f)."""
    n = 1 << logn
    batch = 3
    rng = np.random.default_rng(logn)
    x = (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(np.complex64)
    for sign in (-1, +1):
        y = oracle.ref_contiguous_fft(x, sign, nthreads=4)
        e = oracle.rel_l2(y, oracle.fft(x, sign)).max()
        assert e < 3e-5, (n, sign, e)


def test_dft_bins_matches_the_direct_dft_and_numpy():
    """The sampled direct DFT (stepped roots re-seeded every 256 terms,
    compensated sums) against the full long-double DFT at small n and
    numpy's FP64 FFT at a length past many re-seeds."""
    rng = np.random.default_rng(3)
    x = rng.standard_normal(1000) + 1j * rng.standard_normal(1000)
    bins = np.arange(1000)
    for sign in (-1, +1):
        got = oracle.dft_bins(x, bins, sign)
        assert np.max(np.abs(got - oracle.dft_ld(x, sign))) < 1e-11
    n = 123457
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    bins = np.array([0, 1, 2, 4097, n // 2, n - 1, 98765])
    ref = np.fft.fft(x)[bins]
    got = oracle.dft_bins(x, bins, -1)
    assert np.max(np.abs(got - ref)) / np.sqrt(n) < 1e-11


def test_conv_compat_follows_the_reference_loops():
    """oracle.conv_compat against a literal 1D restatement of the loops of
    Convolution2D_FFT::convolve (Convolution.h:95-148) in long double: the
    kernel written at (x + (K+1)/2) % width (:113-120), the product of the
    spectra (with the conjugate for correlation, :125-137), and the first L
    samples of the inverse scaled by 1 / (width * K^[0]) (:141-148); the
    spectra are taken as direct DFTs."""
    rng = np.random.default_rng(5)
    for L, K in [(4, 1), (5, 1), (7, 3), (8, 2), (13, 6), (16, 16), (1, 4), (2, 5), (3, 11), (6, 30)]:
        s = rng.standard_normal(L)
        h = np.abs(rng.standard_normal(K)) + 0.1
        width = 1
        while width < L + K - 1:
            width *= 2
        width = max(width, 2)
        data = np.zeros(width, np.clongdouble)
        data[:L] = s
        kern = np.zeros(width, np.clongdouble)
        off = (K + 1) // 2
        for x in range(width):
            src = (x + off) % width
            kern[x] = h[src] if src < K else 0
        q = np.arange(width)
        W = np.exp(-2j * np.pi * np.outer(q, q).astype(np.longdouble) / width)
        D, H = W @ data, W @ kern
        for correlate in (False, True):
            prod = D * (np.conj(H) if correlate else H)
            inv = (np.conj(W) @ prod).real / (width * H[0].real)
            ref = oracle.conv_compat(s, h, correlate)
            assert np.allclose(ref, inv[:L].astype(np.float64), rtol=1e-12, atol=1e-12), (L, K, correlate)
