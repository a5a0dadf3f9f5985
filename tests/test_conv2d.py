"""2D FFT convolution (Convolution2D_FFT::convolve, Convolution.h:95-148).

* Oracle pins: the FP64 FFT convolution equals the long-double direct 2D
  convolution and scipy's; the reference-compatible result equals the direct
  convolution shifted by the kernel centre ((kw+1)/2, (kh+1)/2) and divided by
  the kernel sum; correlation equals numpy's (pocketfft) circular correlation.
* Emulator (CPU): the CUDA kernels' index code (conv2d_core.cuh) against the
  oracle, every row tile width and column tile height class.
* GPU: estl_conv2d_* through the C ABI against the oracle.

Tolerance: relative L2 over each image, 1e-6 (FP32 FFTs against FP64).
"""
import ctypes

import numpy as np
import pytest

import oracle

TOL = 1e-6
COMPAT = 2
CORRELATE = 1


def rel(y, ref):
    return float(np.sqrt(np.sum((np.asarray(y, np.float64) - ref) ** 2) / np.sum(ref ** 2)))


def images(count, h, w, seed):
    return np.random.default_rng(seed).standard_normal((count, h, w)).astype(np.float32)


def kernel(kh, kw, seed, positive=False):
    rng = np.random.default_rng(seed)
    k = rng.uniform(0.1, 1.0, (kh, kw)) if positive else rng.standard_normal((kh, kw))
    return k.astype(np.float32)


def expect(a, k, flags):
    return oracle.conv2d_fft(a.astype(np.float64), k.astype(np.float64), correlate=bool(flags & CORRELATE),
                             compat=bool(flags & COMPAT))


# ---------------------------------------------------------------------------
# oracle pins
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("h,w,kh,kw", [(1, 1, 1, 1), (13, 17, 5, 4), (8, 8, 8, 8), (3, 40, 7, 1), (30, 2, 1, 9)])
def test_oracle_matches_direct(h, w, kh, kw):
    a = np.random.default_rng(h * w).standard_normal((h, w))
    k = np.random.default_rng(kh * kw + 1).standard_normal((kh, kw))
    d = oracle.conv2d_direct(a, k)
    assert np.abs(oracle.conv2d_fft(a, k) - d).max() < 1e-12 * max(1.0, np.abs(d).max())
    sig = pytest.importorskip("scipy.signal")
    assert np.abs(sig.convolve2d(a, k) - d).max() < 1e-12 * max(1.0, np.abs(d).max())


@pytest.mark.parametrize("h,w,kh,kw", [(13, 17, 5, 4), (9, 9, 3, 3), (20, 6, 6, 2)])
def test_oracle_compat_is_centred_direct(h, w, kh, kw):
    """Convolution.h:113-120 reads the kernel from ((x + xOffs) mod W,
    (y + yOffs) mod H): the result is the linear convolution shifted by
    (xOffs, yOffs), divided by K^[0] = sum of the kernel (:141-143)."""
    a = np.random.default_rng(3).standard_normal((h, w))
    k = np.random.default_rng(4).uniform(0.1, 1.0, (kh, kw))
    full = np.zeros((h + kh + 2, w + kw + 2))
    d = oracle.conv2d_direct(a, k)
    full[:d.shape[0], :d.shape[1]] = d
    xo, yo = (kw + 1) // 2, (kh + 1) // 2
    ref = full[yo:yo + h, xo:xo + w] / k.sum()
    assert np.abs(oracle.conv2d_fft(a, k, compat=True) - ref).max() < 1e-12


def test_oracle_correlation_matches_numpy():
    a = np.random.default_rng(5).standard_normal((11, 14))
    k = np.random.default_rng(6).standard_normal((4, 6))
    H, W = 16, 32
    A = np.zeros((H, W))
    A[:11, :14] = a
    K = np.zeros((H, W))
    K[:4, :6] = k
    circ = np.real(np.fft.ifft2(np.fft.fft2(A) * np.conj(np.fft.fft2(K))))
    assert np.abs(oracle.conv2d_fft(a, k, correlate=True) - circ[:14, :19]).max() < 1e-12


# ---------------------------------------------------------------------------
# emulator
# ---------------------------------------------------------------------------
def emu_conv2d(emu, imgs, k, flags):
    count, h, w = imgs.shape
    kh, kw = k.shape
    oh, ow = (h, w) if flags & COMPAT else (h + kh - 1, w + kw - 1)
    out = np.full((count, oh, ow), np.nan, np.float32)
    err = ctypes.create_string_buffer(512)
    rc = emu.emu_conv2d_run(w, h, kw, kh, count, flags, imgs.ctypes.data, k.ctypes.data, out.ctypes.data, err,
                            len(err))
    assert rc == 0, err.value.decode()
    return out


# (h, w, kh, kw): padded widths 2^1..2^11 and heights 2^1..2^10, narrow and
# wide arrays, filters larger than the image
SHAPES_EMU = [(1, 1, 1, 1), (2, 3, 1, 1), (5, 3, 3, 2), (12, 20, 5, 5), (40, 9, 9, 40), (3, 100, 2, 29),
              (100, 3, 29, 2), (33, 70, 32, 60), (200, 50, 57, 15), (17, 1000, 4, 25), (520, 6, 5, 3)]


@pytest.mark.parametrize("shape", SHAPES_EMU)
def test_emulated_conv2d(emu, shape):
    h, w, kh, kw = shape
    imgs = images(2, h, w, h + w)
    k = kernel(kh, kw, kh + kw)
    out = emu_conv2d(emu, imgs, k, 0)
    for i in range(2):
        assert rel(out[i], expect(imgs[i], k, 0)) < TOL, shape


@pytest.mark.parametrize("flags", [CORRELATE, COMPAT, COMPAT | CORRELATE])
def test_emulated_conv2d_flags(emu, flags):
    for h, w, kh, kw in [(12, 20, 5, 5), (40, 9, 9, 40), (33, 70, 32, 60)]:
        imgs = images(2, h, w, 7)
        k = kernel(kh, kw, 8, positive=True)
        out = emu_conv2d(emu, imgs, k, flags)
        for i in range(2):
            assert rel(out[i], expect(imgs[i], k, flags)) < TOL, (flags, h, w, kh, kw)


def test_emulated_conv2d_rejects(emu):
    err = ctypes.create_string_buffer(512)
    z = np.zeros(4, np.float32)
    # padded height 2^13 > 2^12
    assert emu.emu_conv2d_run(4, 5000, 1, 4000, 1, 0, z.ctypes.data, z.ctypes.data, z.ctypes.data, err, 512) == 2
    assert emu.emu_conv2d_run(0, 4, 1, 1, 1, 0, z.ctypes.data, z.ctypes.data, z.ctypes.data, err, 512) == 2


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def gpu_conv2d(engine, imgs, k, flags, stream=None):
    import torch
    count, h, w = imgs.shape
    kh, kw = k.shape
    p = engine.Conv2DPlan(w, h, kw, kh, count, flags)
    p.set_filter(torch.from_numpy(np.ascontiguousarray(k)).cuda(), stream=stream)
    out = p.execute(torch.from_numpy(np.ascontiguousarray(imgs)).cuda(), stream=stream)
    torch.cuda.synchronize()
    res = out.cpu().numpy()
    p.close()
    return res


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES_EMU + [(512, 512, 31, 31), (1000, 1500, 25, 49), (2048, 4096, 17, 33),
                                                (3000, 9000, 64, 100)])
def test_gpu_conv2d(engine, shape):
    h, w, kh, kw = shape
    count = 3 if h * w <= (1 << 20) else 1
    imgs = images(count, h, w, h + w)
    k = kernel(kh, kw, kh + kw)
    out = gpu_conv2d(engine, imgs, k, 0)
    for i in range(count):
        assert rel(out[i], expect(imgs[i], k, 0)) < TOL, shape


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [CORRELATE, COMPAT, COMPAT | CORRELATE])
def test_gpu_conv2d_flags(engine, flags):
    for h, w, kh, kw in [(12, 20, 5, 5), (200, 50, 57, 15), (700, 900, 31, 17)]:
        imgs = images(2, h, w, 9)
        k = kernel(kh, kw, 10, positive=True)
        out = gpu_conv2d(engine, imgs, k, flags)
        for i in range(2):
            assert rel(out[i], expect(imgs[i], k, flags)) < TOL, (flags, h, w, kh, kw)


@pytest.mark.gpu
def test_gpu_conv2d_errors(engine):
    import torch
    from estl_gb300 import EstlError
    with pytest.raises(EstlError) as e:
        engine.Conv2DPlan(4, 5000, 1, 4000)  # pads to 2^13 rows
    assert e.value.name == "ESTL_UNSUPPORTED_SIZE"
    with pytest.raises(EstlError):
        engine.Conv2DPlan(0, 4, 1, 1)
    p = engine.Conv2DPlan(8, 8, 3, 3)
    with pytest.raises(EstlError):  # filter not set
        p.execute(torch.zeros(64, device="cuda"))
    with pytest.raises(EstlError):  # wrong filter size
        p.set_filter(torch.zeros(8, device="cuda"))
    from estl_gb300._lib import lib
    k = torch.zeros(16, device="cuda")
    # a float pointer off its 4-byte boundary is refused before any launch
    assert lib().estl_conv2d_plan_set_filter(p._h, ctypes.c_void_p(k.data_ptr() + 2), None) != 0
    p.set_filter(k[:9])
    x = torch.zeros(200, device="cuda")
    assert lib().estl_conv2d_plan_execute(p._h, ctypes.c_void_p(x.data_ptr() + 1),
                                          ctypes.c_void_p(x.data_ptr() + 128), None) != 0
    p.close()
