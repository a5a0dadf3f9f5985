"""Oracle package — TEST INFRASTRUCTURE ONLY.

The reference results the FFT engine is tested against, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline`` leg and
the ``--impl reference`` arm) may import it.

* ``fft`` / ``dft_ld`` / ``conv_fft`` / ``conv_direct`` / ``conv2d_fft`` /
  ``conv2d_direct``: FP64 restatement of the reference's CPU transform
  (``FFT_FFTW3.h:23-31``, plan semantics of ``fftwf_plan_many_dft``) and of its
  FFT convolution (``Convolution.h:95-148``, in 1D and in 2D), in ``oracle.c``.
* ``ref_contiguous_fft``: FP32 restatement of the reference's own GPU
  algorithm (``FFT_OpenCL_Contiguous.h:144-184``), in ``ref_contiguous.c``;
  timed as the CPU baseline.

Parity pins: the known-answer test of ``tests/Test.cpp:60-77`` (cosine in,
two spikes of M/2 out), a long-double direct DFT and ``numpy.fft`` — see
``tests/test_oracle.py``.
"""
import ctypes
import os
import subprocess

import numpy as np

_DIR = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_DIR, "_build")
_LIB_PATH = os.path.join(_BUILD, "liboracle.so")
_SOURCES = ["oracle.c", "ref_contiguous.c"]
_lib = None


def build(force=False):
    """Compile oracle.c and ref_contiguous.c into _build/liboracle.so (gcc)."""
    srcs = [os.path.join(_DIR, s) for s in _SOURCES]
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(s) for s in srcs)):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-pthread", "-o", _LIB_PATH] + srcs + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        lib.oracle_fft.argtypes = [P, P, I64, I64, ctypes.c_int, ctypes.c_int]
        lib.oracle_fft.restype = ctypes.c_int
        lib.oracle_dft_ld.argtypes = [P, P, I64, ctypes.c_int]
        lib.oracle_dft_bins.argtypes = [P, P, I64, P, I64, ctypes.c_int]
        lib.oracle_conv_direct.argtypes = [P, I64, P, I64, P]
        lib.oracle_conv_fft.argtypes = [P, I64, P, I64, P, ctypes.c_int]
        lib.oracle_conv_fft.restype = ctypes.c_int
        lib.oracle_conv_circular.argtypes = [P, I64, P, I64, I64, P, I64, ctypes.c_int]
        lib.oracle_conv_circular.restype = ctypes.c_int
        lib.oracle_conv2d_fft.argtypes = [P, I64, I64, P, I64, I64, P, ctypes.c_int, ctypes.c_int]
        lib.oracle_conv2d_fft.restype = ctypes.c_int
        lib.oracle_conv2d_direct.argtypes = [P, I64, I64, P, I64, I64, P]
        lib.ref_contiguous_fft.argtypes = [P, P, P, I64, I64, ctypes.c_int, ctypes.c_int]
        lib.ref_contiguous_fft.restype = ctypes.c_int
        _lib = lib
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def fft(x, sign=-1, nthreads=None):
    """FP64 batched FFT along the last axis (power-of-two length).

    sign -1 = FFTW_FORWARD (exp(-2 pi i jk/n)), +1 = FFTW_BACKWARD; unnormalised.
    Returns complex128 with the shape of x.
    """
    x = np.ascontiguousarray(x, dtype=np.complex128)
    n = x.shape[-1]
    batch = x.size // n if n else 0
    out = np.empty_like(x)
    if nthreads is None:
        nthreads = min(os.cpu_count() or 1, 64)
    rc = _load().oracle_fft(_ptr(x), _ptr(out), n, batch, int(sign), int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle_fft: unsupported length {n}")
    return out


def dft_ld(x, sign=-1):
    """Long-double direct DFT of one 1-D sequence (O(n^2), for small n)."""
    x = np.ascontiguousarray(x, dtype=np.complex128).ravel()
    out = np.empty_like(x)
    _load().oracle_dft_ld(_ptr(x), _ptr(out), x.size, int(sign))
    return out


def dft_bins(x, bins, sign=-1):
    """Bins `bins` of the direct DFT of one 1-D sequence of any length (O(n)
    per bin; exactly reduced angles, roots re-seeded from long double,
    compensated double sums): a reference independent of any FFT for long
    transforms sampled at a few frequencies."""
    x = np.ascontiguousarray(x, dtype=np.complex128).ravel()
    bins = np.ascontiguousarray(bins, dtype=np.int64).ravel()
    out = np.empty(bins.size, np.complex128)
    _load().oracle_dft_bins(_ptr(x), _ptr(out), x.size, _ptr(bins), bins.size, int(sign))
    return out


def conv_direct(a, b):
    """Long-double direct linear convolution of two real sequences."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.empty(a.size + b.size - 1)
    _load().oracle_conv_direct(_ptr(a), a.size, _ptr(b), b.size, _ptr(out))
    return out


def conv_fft(a, b, correlate=False):
    """FP64 FFT linear convolution (zero-padded to the next power of two)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.empty(a.size + b.size - 1)
    _load().oracle_conv_fft(_ptr(a), a.size, _ptr(b), b.size, _ptr(out), int(bool(correlate)))
    return out


def conv_circular(a, b, n, correlate=False):
    """FP64 n-point circular convolution (correlation: product with the
    conjugate spectrum) of two real sequences zero-padded to n."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.empty(n)
    rc = _load().oracle_conv_circular(_ptr(a), a.size, _ptr(b), b.size, int(n), _ptr(out), int(n), int(bool(correlate)))
    if rc:
        raise ValueError("n must cover both sequences")
    return out


def conv_compat(s, h, correlate=False):
    """1D restatement of Convolution2D_FFT::convolve's own result
    (Convolution.h:95-148): both padded to n = nextPowerOf2(L + K - 1) (at
    least 2, the engine's smallest transform; the padding beyond L + K - 1
    holds zeros either way), the kernel shifted cyclically by (K + 1) / 2
    (:113-120), so output m is circular sample (m + (K + 1) / 2) mod n of the
    convolution -- of the correlation, whose spectrum is conjugated after the
    shift (:125-137), sample (m - (K + 1) / 2) mod n -- divided by
    sum(h) = K^[0] (:141-143), L samples kept (:146-148)."""
    L, K = len(s), len(h)
    n = 2
    while n < L + K - 1:
        n *= 2
    circ = conv_circular(s, h, n, correlate)
    off = -((K + 1) // 2) if correlate else (K + 1) // 2
    return circ[(np.arange(L) + off) % n] / np.sum(np.asarray(h, np.float64))


def conv2d_fft(a, k, correlate=False, compat=False):
    """FP64 2D FFT convolution of a real image (h, w) with a real kernel
    (kh, kw), after Convolution2D_FFT::convolve (Convolution.h:95-148):
    compat=False gives the full linear convolution (h+kh-1, w+kw-1) / 1;
    compat=True the reference's centred, K^[0]-normalised (h, w) result."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    k = np.ascontiguousarray(k, dtype=np.float64)
    h, w = a.shape
    kh, kw = k.shape
    shape = (h, w) if compat else (h + kh - 1, w + kw - 1)
    out = np.empty(shape)
    _load().oracle_conv2d_fft(_ptr(a), h, w, _ptr(k), kh, kw, _ptr(out), int(bool(correlate)), int(bool(compat)))
    return out


def conv2d_direct(a, k):
    """Long-double direct 2D linear convolution, shape (h+kh-1, w+kw-1)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    k = np.ascontiguousarray(k, dtype=np.float64)
    h, w = a.shape
    kh, kw = k.shape
    out = np.empty((h + kh - 1, w + kw - 1))
    _load().oracle_conv2d_direct(_ptr(a), h, w, _ptr(k), kh, kw, _ptr(out))
    return out


def ref_contiguous_fft(x, sign=-1, nthreads=None):
    """FP32 restatement of FFT_OpenCL_Contiguous on the host cores."""
    x = np.ascontiguousarray(x, dtype=np.complex64)
    n = x.shape[-1]
    batch = x.size // n
    out = np.empty_like(x)
    work = np.empty_like(x)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    rc = _load().ref_contiguous_fft(_ptr(x), _ptr(out), _ptr(work), n, batch, int(sign), int(nthreads))
    if rc != 0:
        raise ValueError(f"ref_contiguous_fft: unsupported length {n}")
    return out


def rel_l2(y, ref):
    """Per-transform relative L2 error sqrt(sum|y-ref|^2 / sum|ref|^2) along the
    last axis (the metric of OpenCL_FFT/main.cpp:333-359, without its division
    by FLT_EPSILON)."""
    y = np.asarray(y, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    num = np.sum(np.abs(y - ref) ** 2, axis=-1)
    den = np.sum(np.abs(ref) ** 2, axis=-1)
    return np.sqrt(num / np.maximum(den, 1e-300))
