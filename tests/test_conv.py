"""FFT convolution (Convolution2D_FFT, Convolution.h:95-154, in 1D and batched).

* emulator (CPU): every size class through the host emulator of the
  convolution kernels, with bounds checks, against the FP64 oracle;
* GPU: the C ABI (estl_conv_execute, estl_conv_plan_*) against the oracle.

Tolerance: rel-L2 of the output vector <= 1e-6 against the FP64 FFT
convolution (itself checked against a long-double direct convolution in
tests/test_oracle.py).
"""
import ctypes

import numpy as np
import pytest

import oracle

TOL = 1e-6


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.sum((a - b) ** 2) / max(np.sum(b ** 2), 1e-300)))


def make_requests(shapes, seed):
    """Packed signals / filters / outputs for (L, K) pairs."""
    rng = np.random.default_rng(seed)
    reqs, sigs, filts = [], [], []
    so = fo = oo = 0
    for L, K in shapes:
        s = rng.standard_normal(L).astype(np.float32)
        f = rng.standard_normal(K).astype(np.float32)
        reqs.append((L, K, so, fo, oo))
        sigs.append(s)
        filts.append(f)
        so += L
        fo += K
        oo += L + K - 1
    return reqs, np.concatenate(sigs), np.concatenate(filts), oo


def compat_reference(s, f, correlate=False):
    """Convolution.h's normalisation and crop in 1D: the kernel shifted
    cyclically by (K+1)/2 (:113-120), divided by sum(h) (= K^[0], :141-143),
    L samples kept (:146-148) -- oracle.conv_compat."""
    return oracle.conv_compat(s, f, correlate)


def emu_conv(emu, reqs, sig, filt, out_len, flags=0, shared=False):
    arr = np.array(reqs, dtype=np.int64).ravel()
    out = np.full(out_len, np.nan, np.float32)
    err = ctypes.create_string_buffer(512)
    rc = emu.emu_conv_run(arr.ctypes.data, len(reqs), flags, int(shared), sig.ctypes.data, filt.ctypes.data,
                          out.ctypes.data, err, len(err))
    assert rc == 0, err.value
    return out


SHAPES_EMU = [(1, 1), (3, 2), (5, 4), (16, 16), (100, 17), (256, 16), (1000, 64), (2000, 100), (4096, 300),
              (9000, 700), (13000, 3000), (20000, 4096)]


def test_emulated_batch_all_size_classes(emu):
    reqs, sig, filt, olen = make_requests(SHAPES_EMU, 1)
    out = emu_conv(emu, reqs, sig, filt, olen)
    for L, K, so, fo, oo in reqs:
        ref = oracle.conv_fft(sig[so:so + L].astype(np.float64), filt[fo:fo + K].astype(np.float64))
        assert rel(out[oo:oo + L + K - 1], ref) < TOL, (L, K)


def test_emulated_correlation_and_compat(emu):
    shapes = [(300, 40), (5000, 33), (20000, 257)]
    reqs, sig, filt, olen = make_requests(shapes, 2)
    out = emu_conv(emu, reqs, sig, filt, olen, flags=1)
    for L, K, so, fo, oo in reqs:
        ref = oracle.conv_fft(sig[so:so + L].astype(np.float64), filt[fo:fo + K].astype(np.float64), correlate=True)
        assert rel(out[oo:oo + L + K - 1], ref) < TOL
    # reference-compatible mode writes L samples per request
    creqs = []
    oo = 0
    for L, K, so, fo, _ in reqs:
        creqs.append((L, K, so, fo, oo))
        oo += L
    # positive filters keep sum(h) away from zero
    filt_pos = np.abs(filt) + 0.1
    out = emu_conv(emu, creqs, sig, filt_pos, oo, flags=2)
    for L, K, so, fo, oo in creqs:
        ref = compat_reference(sig[so:so + L], filt_pos[fo:fo + K])
        assert rel(out[oo:oo + L], ref) < TOL


def test_emulated_shared_filter(emu):
    L, K, n = 3000, 100, 7
    rng = np.random.default_rng(3)
    sig = rng.standard_normal(L * n).astype(np.float32)
    filt = rng.standard_normal(K).astype(np.float32)
    reqs = [(L, K, i * L, 0, i * (L + K - 1)) for i in range(n)]
    out = emu_conv(emu, reqs, sig, filt, n * (L + K - 1), shared=True)
    for i in range(n):
        ref = oracle.conv_fft(sig[i * L:(i + 1) * L].astype(np.float64), filt.astype(np.float64))
        assert rel(out[i * (L + K - 1):(i + 1) * (L + K - 1)], ref) < TOL


NO_PAIRING = 4
COMPLEX = 8


@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_emulated_pairs_odd_buckets(emu, flags):
    """Two real requests per complex transform (the default for n <= 2^14):
    buckets of one, two, three and five requests of different lengths (odd
    buckets leave an unpaired last request), every flag combination, paired
    and unpaired (ESTL_CONV_NO_PAIRING), against the oracle."""
    shapes = [(700, 90), (1000, 20), (600, 300), (900, 60), (1020, 5),  # n = 1024: five requests
              (3000, 1000), (2500, 1597),                                # n = 4096: two
              (9000, 700), (12000, 300), (8500, 2),                      # n = 16384: three
              (40, 9)]                                                   # n = 64: one
    reqs, sig, filt, _ = make_requests(shapes, 21)
    compat = bool(flags & 2)
    if compat:
        filt = np.abs(filt) + 0.1
    creqs, oo = [], 0
    for L, K, so, fo, _ in reqs:
        creqs.append((L, K, so, fo, oo))
        oo += L if compat else L + K - 1
    outs = [emu_conv(emu, creqs, sig, filt, oo, flags=flags | extra) for extra in (0, NO_PAIRING)]
    for L, K, so, fo, o in creqs:
        s, f = sig[so:so + L], filt[fo:fo + K]
        if compat:
            ref = compat_reference(s, f, correlate=bool(flags & 1))
        else:
            ref = oracle.conv_fft(s.astype(np.float64), f.astype(np.float64), correlate=bool(flags & 1))
        n_out = L if compat else L + K - 1
        for out in outs:
            assert rel(out[o:o + n_out], ref) < TOL, (flags, L, K)


def test_emulated_pairs_disparate_magnitudes(emu):
    """Paired requests whose outputs differ by many orders of magnitude (a
    2-tap filter beside a 700-tap one, signals scaled by 1e4 and 1e-3,
    filters by 1e-3 and 1e2): the power-of-two balancing keeps every request
    at the FP32 tolerance of its own magnitude."""
    shapes = [(8500, 2), (9000, 700), (8000, 300), (3000, 5), (3000, 1000)]
    reqs, sig, filt, olen = make_requests(shapes, 31)
    scale_s = [1e4, 1.0, 1e-3, 1.0, 1e3]
    scale_f = [1.0, 1e-3, 1.0, 1e2, 1.0]
    for (L, K, so, fo, _), a, b in zip(reqs, scale_s, scale_f):
        sig[so:so + L] *= np.float32(a)
        filt[fo:fo + K] *= np.float32(b)
    out = emu_conv(emu, reqs, sig, filt, olen)
    for L, K, so, fo, oo in reqs:
        ref = oracle.conv_fft(sig[so:so + L].astype(np.float64), filt[fo:fo + K].astype(np.float64))
        assert rel(out[oo:oo + L + K - 1], ref) < TOL, (L, K)


def test_emulated_pairs_shared_filter(emu):
    """One filter for every request (the convolution plan): pairs multiply by
    the plain spectrum H; odd and even counts."""
    for n in (6, 7):
        L, K = 5000, 77
        rng = np.random.default_rng(n)
        sig = rng.standard_normal(L * n).astype(np.float32)
        filt = rng.standard_normal(K).astype(np.float32)
        reqs = [(L, K, i * L, 0, i * (L + K - 1)) for i in range(n)]
        out = emu_conv(emu, reqs, sig, filt, n * (L + K - 1), shared=True)
        for i in range(n):
            ref = oracle.conv_fft(sig[i * L:(i + 1) * L].astype(np.float64), filt.astype(np.float64))
            assert rel(out[i * (L + K - 1):(i + 1) * (L + K - 1)], ref) < TOL


SPLIT_TOL = {1: TOL, 2: 2e-5, 3: TOL}


@pytest.mark.parametrize("split", [1, 2, 3])
def test_emulated_split_precision(emu, split):
    """Convolutions whose FFT stages run the split-precision tensor-core tiles
    (precision in bits 8-9 of the flags): fp16 hi+lo and bf16 hi+mid+lo keep
    the 1e-6 target, bf16 hi+lo (16 significant bits) stays within 2e-5."""
    reqs, sig, filt, olen = make_requests(SHAPES_EMU, 11)
    out = emu_conv(emu, reqs, sig, filt, olen, flags=split << 8)
    for L, K, so, fo, oo in reqs:
        ref = oracle.conv_fft(sig[so:so + L].astype(np.float64), filt[fo:fo + K].astype(np.float64))
        assert rel(out[oo:oo + L + K - 1], ref) < SPLIT_TOL[split], (split, L, K)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def gpu_conv_batch(engine, reqs, sig, filt, out_len, flags=0):
    import torch

    from estl_gb300._lib import ConvRequest, check, lib
    L = lib()
    arr = (ConvRequest * len(reqs))(*[ConvRequest(*r) for r in reqs])
    ws = ctypes.c_size_t()
    check(L.estl_conv_workspace_size(arr, len(reqs), flags, ctypes.byref(ws)))
    d_sig = torch.from_numpy(sig).cuda()
    d_filt = torch.from_numpy(filt).cuda()
    d_out = torch.full((out_len,), float("nan"), device="cuda")
    d_ws = torch.empty(ws.value + 256, dtype=torch.uint8, device="cuda")
    base = (d_ws.data_ptr() + 255) // 256 * 256
    st = torch.cuda.current_stream().cuda_stream
    check(L.estl_conv_execute(arr, len(reqs), flags, ctypes.c_void_p(d_sig.data_ptr()),
                              ctypes.c_void_p(d_filt.data_ptr()), ctypes.c_void_p(d_out.data_ptr()),
                              ctypes.c_void_p(base), ws.value, ctypes.c_void_p(st)))
    return d_out.cpu().numpy()


@pytest.mark.gpu
def test_gpu_batch_mixed_sizes(engine):
    shapes = SHAPES_EMU + [(1 << 16, 4096), (1 << 18, 1000), ((1 << 20) - 7, 4096), (1 << 20, 4096)]
    reqs, sig, filt, olen = make_requests(shapes, 4)
    out = gpu_conv_batch(engine, reqs, sig, filt, olen)
    for L, K, so, fo, oo in reqs:
        ref = oracle.conv_fft(sig[so:so + L].astype(np.float64), filt[fo:fo + K].astype(np.float64))
        assert rel(out[oo:oo + L + K - 1], ref) < TOL, (L, K)


@pytest.mark.gpu
def test_gpu_correlation_and_compat(engine):
    shapes = [(300, 40), (5000, 33), (20000, 257), (300000, 2049)]
    reqs, sig, filt, olen = make_requests(shapes, 5)
    out = gpu_conv_batch(engine, reqs, sig, filt, olen, flags=1)
    for L, K, so, fo, oo in reqs:
        ref = oracle.conv_fft(sig[so:so + L].astype(np.float64), filt[fo:fo + K].astype(np.float64), correlate=True)
        assert rel(out[oo:oo + L + K - 1], ref) < TOL
    creqs, oo = [], 0
    for L, K, so, fo, _ in reqs:
        creqs.append((L, K, so, fo, oo))
        oo += L
    filt_pos = np.abs(filt) + 0.1
    out = gpu_conv_batch(engine, creqs, sig, filt_pos, oo, flags=2)
    for L, K, so, fo, oo in creqs:
        assert rel(out[oo:oo + L], compat_reference(sig[so:so + L], filt_pos[fo:fo + K])) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [2, 3])
def test_gpu_compat_correlation_and_wrapped_crop(engine, flags):
    """Reference-compatible mode on the GPU: correlation (the output shifted the
    other way, the conjugate taken after the kernel shift) and crops that wrap
    (a 1-tap filter on power-of-two signals), through the paired and unpaired
    single tiles and the real-input and complex four-step forms, against
    oracle.conv_compat (pinned to a restatement of Convolution.h:95-148)."""
    shapes = [(4, 1), (16, 1), (1024, 1), (16384, 1), (32768, 1), (5, 1), (300, 40), (5000, 33), (20000, 257)]
    reqs, sig, filt, _ = make_requests(shapes, 73)
    filt = np.abs(filt) + 0.1
    creqs, oo = [], 0
    for L, K, so, fo, _ in reqs:
        creqs.append((L, K, so, fo, oo))
        oo += L
    for extra in (0, NO_PAIRING, COMPLEX):
        out = gpu_conv_batch(engine, creqs, sig, filt, oo, flags=flags | extra)
        for L, K, so, fo, o in creqs:
            ref = compat_reference(sig[so:so + L], filt[fo:fo + K], correlate=bool(flags & 1))
            assert rel(out[o:o + L], ref) < TOL, (L, K, flags, extra)


@pytest.mark.gpu
@pytest.mark.parametrize("L,K,count", [(1000, 31, 64), (50000, 1000, 8), (1 << 20, 4096, 2)])
def test_gpu_conv_plan(engine, L, K, count):
    import torch

    from estl_gb300._lib import check, lib
    Lb = lib()
    plan = ctypes.c_void_p()
    check(Lb.estl_conv_plan_create(L, K, count, 0, ctypes.byref(plan)))
    try:
        rng = np.random.default_rng(L + K)
        sig = rng.standard_normal(L * count).astype(np.float32)
        filt = rng.standard_normal(K).astype(np.float32)
        olen = int(Lb.estl_conv_output_length(L, K, 0))
        st = torch.cuda.current_stream().cuda_stream
        d_filt = torch.from_numpy(filt).cuda()
        check(Lb.estl_conv_plan_set_filter(plan, ctypes.c_void_p(d_filt.data_ptr()), ctypes.c_void_p(st)))
        d_sig = torch.from_numpy(sig).cuda()
        d_out = torch.full((olen * count,), float("nan"), device="cuda")
        for _ in range(2):  # cached spectrum reused
            check(Lb.estl_conv_plan_execute(plan, ctypes.c_void_p(d_sig.data_ptr()),
                                            ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(st)))
        out = d_out.cpu().numpy()
        for i in range(count):
            ref = oracle.conv_fft(sig[i * L:(i + 1) * L].astype(np.float64), filt.astype(np.float64))
            assert rel(out[i * olen:(i + 1) * olen], ref) < TOL
    finally:
        Lb.estl_conv_plan_destroy(plan)


@pytest.mark.gpu
@pytest.mark.parametrize("split", [1, 2, 3])
def test_gpu_split_precision(engine, split):
    shapes = SHAPES_EMU + [(1 << 16, 4096), ((1 << 20) - 7, 4096)]
    reqs, sig, filt, olen = make_requests(shapes, 12)
    out = gpu_conv_batch(engine, reqs, sig, filt, olen, flags=split << 8)
    for L, K, so, fo, oo in reqs:
        ref = oracle.conv_fft(sig[so:so + L].astype(np.float64), filt[fo:fo + K].astype(np.float64))
        assert rel(out[oo:oo + L + K - 1], ref) < SPLIT_TOL[split], (split, L, K)


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [0, NO_PAIRING, 1 << 8, (1 << 8) | NO_PAIRING, 3 << 8])
def test_gpu_pairs(engine, flags):
    """Paired (default) and unpaired single-tile convolutions, FP32 and split
    precision, odd buckets, against the oracle."""
    shapes = [(700, 90), (1000, 20), (600, 300), (900, 60), (1020, 5), (3000, 1000), (2500, 1597),
              (9000, 700), (12000, 300), (8500, 2), (40, 9)] * 3
    reqs, sig, filt, olen = make_requests(shapes, 22)
    for i, (L, K, so, fo, _) in enumerate(reqs):  # magnitudes over eight decades
        sig[so:so + L] *= np.float32(10.0 ** ((i % 5) - 2))
        filt[fo:fo + K] *= np.float32(10.0 ** (2 - (i % 4)))
    out = gpu_conv_batch(engine, reqs, sig, filt, olen, flags=flags)
    tol = SPLIT_TOL.get(flags >> 8, TOL)
    for L, K, so, fo, oo in reqs:
        ref = oracle.conv_fft(sig[so:so + L].astype(np.float64), filt[fo:fo + K].astype(np.float64))
        assert rel(out[oo:oo + L + K - 1], ref) < tol, (flags, L, K)


def test_emulated_request_validation(emu):
    """Requests are checked before any work: lengths >= 1, offsets >= 0,
    lengths and offsets at most 2^40 (no 64-bit sum overflows), padded length
    at most the supported maximum."""
    z = np.zeros(8, np.float32)
    err = ctypes.create_string_buffer(512)
    bad = [(0, 4, 0, 0, 0), (8, 4, -1, 0, 0), ((1 << 62), 4, 0, 0, 0), (8, (1 << 62), 0, 0, 0),
           (8, 4, 0, 0, (1 << 62)), ((1 << 30), 4, 0, 0, 0)]
    for r in bad:
        arr = np.array([r], dtype=np.int64).ravel()
        rc = emu.emu_conv_run(arr.ctypes.data, 1, 0, 0, z.ctypes.data, z.ctypes.data, z.ctypes.data, err, len(err))
        assert rc == 2 and err.value, r


@pytest.mark.parametrize("flags", [0, 1, 2])
def test_emulated_real_input_four_step(emu, flags):
    """Padded lengths above 2^14 run the real-input four-step form (each real
    request as an N/2-point complex transform, the spectrum split through
    mirrored row pairs): 2^15, 2^16 and 2^17, convolution, correlation and
    the reference-compatible mode, against the oracle and bit-for-bit
    the complex form (ESTL_CONV_COMPLEX) within the tolerance."""
    shapes = [(20000, 700), (16384, 2), (40000, 100), (70000, 33)]
    reqs, sig, filt, _ = make_requests(shapes, 31)
    compat = bool(flags & 2)
    if compat:
        filt = np.abs(filt) + 0.1
    creqs, oo = [], 0
    for L, K, so, fo, _ in reqs:
        creqs.append((L, K, so, fo, oo))
        oo += L if compat else L + K - 1
    half = emu_conv(emu, creqs, sig, filt, oo, flags=flags)
    full = emu_conv(emu, creqs, sig, filt, oo, flags=flags | COMPLEX)
    for L, K, so, fo, o in creqs:
        s, f = sig[so:so + L], filt[fo:fo + K]
        if compat:
            ref, n = compat_reference(s, f, correlate=bool(flags & 1)), L
        else:
            ref, n = oracle.conv_fft(s.astype(np.float64), f.astype(np.float64), correlate=bool(flags & 1)), L + K - 1
        assert rel(half[o:o + n], ref) < TOL, (L, K, flags)
        assert rel(full[o:o + n], ref) < TOL, (L, K, flags)


@pytest.mark.parametrize("flags", [2, 3])
def test_emulated_compat_crop_wraps(emu, flags):
    """Reference-compatible mode when the crop runs past the padded length:
    a 1-tap filter on a power-of-two signal pads to n = L, so the kernel's
    cyclic shift by (K+1)/2 = 1 (Convolution.h:113-120) makes the last output
    sample circular sample 0.  Single-tile (paired and unpaired), real-input
    four-step and complex four-step paths."""
    shapes = [(4, 1), (16, 1), (1024, 1), (16384, 1), (32768, 1), (5, 1)]
    reqs, sig, filt, _ = make_requests(shapes, 71)
    filt = np.abs(filt) + 0.1
    creqs, oo = [], 0
    for L, K, so, fo, _ in reqs:
        creqs.append((L, K, so, fo, oo))
        oo += L
    for extra in (0, NO_PAIRING, COMPLEX):
        out = emu_conv(emu, creqs, sig, filt, oo, flags=flags | extra)
        for L, K, so, fo, o in creqs:
            ref = compat_reference(sig[so:so + L], filt[fo:fo + K], correlate=bool(flags & 1))
            assert rel(out[o:o + L], ref) < TOL, (L, K, flags, extra)


@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_emulated_filter_longer_than_signal(emu, flags):
    """Filters longer than their signals (K > L), from 1 sample against 5 taps
    to 500 samples against 20000 taps (padded 2^15: the real-input
    four-step): full convolution and correlation (L + K - 1 samples) and the
    reference-compatible mode (L samples of the kernel-shifted circular
    result), paired, unpaired and complex, against the oracle."""
    shapes = [(1, 5), (3, 40), (100, 1000), (50, 3000), (700, 9000), (500, 20000)]
    reqs, sig, filt, _ = make_requests(shapes, 101 + flags)
    compat = bool(flags & 2)
    if compat:
        filt = np.abs(filt) + 0.1
    creqs, oo = [], 0
    for L, K, so, fo, _ in reqs:
        creqs.append((L, K, so, fo, oo))
        oo += L if compat else L + K - 1
    for extra in (0, NO_PAIRING, COMPLEX):
        out = emu_conv(emu, creqs, sig, filt, oo, flags=flags | extra)
        for L, K, so, fo, o in creqs:
            s, f = sig[so:so + L], filt[fo:fo + K]
            if compat:
                ref, n = compat_reference(s, f, correlate=bool(flags & 1)), L
            else:
                ref = oracle.conv_fft(s.astype(np.float64), f.astype(np.float64), correlate=bool(flags & 1))
                n = L + K - 1
            assert rel(out[o:o + n], ref) < TOL, (L, K, flags, extra)


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_gpu_filter_longer_than_signal(engine, flags):
    """K > L on the GPU through estl_conv_execute, up to a 4000-sample signal
    against a 200000-tap filter (padded 2^18), every mode and form, against
    the oracle."""
    shapes = [(1, 5), (3, 40), (100, 1000), (50, 3000), (700, 9000), (500, 20000), (4000, 200000)]
    reqs, sig, filt, _ = make_requests(shapes, 111 + flags)
    compat = bool(flags & 2)
    if compat:
        filt = np.abs(filt) + 0.1
    creqs, oo = [], 0
    for L, K, so, fo, _ in reqs:
        creqs.append((L, K, so, fo, oo))
        oo += L if compat else L + K - 1
    for extra in (0, NO_PAIRING, COMPLEX):
        out = gpu_conv_batch(engine, creqs, sig, filt, oo, flags=flags | extra)
        for L, K, so, fo, o in creqs:
            s, f = sig[so:so + L], filt[fo:fo + K]
            if compat:
                ref, n = compat_reference(s, f, correlate=bool(flags & 1)), L
            else:
                ref = oracle.conv_fft(s.astype(np.float64), f.astype(np.float64), correlate=bool(flags & 1))
                n = L + K - 1
            assert rel(out[o:o + n], ref) < TOL, (L, K, flags, extra)
