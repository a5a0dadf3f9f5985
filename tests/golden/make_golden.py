"""Generates tests/golden/dft_golden.npz: seeded inputs and their DFTs computed
with mpmath at 40 significant digits (independent of the C oracle).

Inputs follow the distributions of the benchmark configurations: re/im
i.i.d. uniform[-1, 1) (the Apple harness distribution, OpenCL_FFT/main.cpp:439-440)
and the known-answer cosine of tests/Test.cpp:60-63; powers of two 1..256 and
the lengths 3, 5, 12, 100, 1000 (the Bluestein path).  Output convention is
FFTW's (FFT_FFTW3.h:26-28): forward exp(-2 pi i jk/n), unnormalised.

Run:  python tests/golden/make_golden.py
"""
import os

import mpmath
import numpy as np

mpmath.mp.dps = 40
HERE = os.path.dirname(os.path.abspath(__file__))


def dft_mp(x, sign):
    n = len(x)
    xs = [mpmath.mpc(float(v.real), float(v.imag)) for v in x]
    w = [mpmath.exp(sign * 2j * mpmath.pi * m / n) for m in range(n)]
    out = np.empty(n, dtype=np.complex128)
    for k in range(n):
        s = mpmath.mpc(0)
        for j in range(n):
            s += xs[j] * w[(j * k) % n]
        out[k] = complex(s)
    return out


def main():
    rng = np.random.default_rng(20111)
    arrays = {}
    for logn in range(0, 9):
        n = 1 << logn
        for sign in (-1, +1):
            x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
            arrays[f"x_{n}_{sign}"] = x
            arrays[f"y_{n}_{sign}"] = dft_mp(x.astype(np.complex128), sign)
    # known-answer input of tests/Test.cpp:62-63 for M = 64, effK = 5
    m, eff = 64, 5
    q = np.arange(m)
    x = np.cos(2 * np.pi * (eff * q) / m).astype(np.float32).astype(np.complex64)
    arrays["kat_x"] = x
    arrays["kat_y"] = dft_mp(x.astype(np.complex128), -1)
    # lengths that are not powers of two (the Bluestein path), own generator so
    # that the arrays above stay as they were
    rng2 = np.random.default_rng(20112)
    for n in (3, 5, 12, 100, 1000):
        for sign in (-1, +1):
            x = (rng2.uniform(-1, 1, n) + 1j * rng2.uniform(-1, 1, n)).astype(np.complex64)
            arrays[f"x_{n}_{sign}"] = x
            arrays[f"y_{n}_{sign}"] = dft_mp(x.astype(np.complex128), sign)
    np.savez_compressed(os.path.join(HERE, "dft_golden.npz"), **arrays)
    print("wrote", len(arrays), "arrays")


if __name__ == "__main__":
    main()
