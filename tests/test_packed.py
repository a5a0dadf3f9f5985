"""Uneven batches: packed transforms of mixed power-of-two lengths with an
offsets array (the uneven-batch configuration: 8192 transforms, lengths
log-uniform over 2^6..2^16, complex N(0,1), seed 3).

* emulator (CPU): both execution modes of the packed kernel (persistent work
  queue; one launch per size) through the bounds-checked host emulator;
* GPU: the C ABI at the full configuration, both modes, against the oracle.
"""
import ctypes
import json

import numpy as np
import pytest

import oracle


def tol(n):
    return 2e-6


def make_batch(count, lo, hi, seed, gap=0):
    rng = np.random.default_rng(seed)
    e = rng.integers(lo, hi + 1, count)
    sizes = (1 << e).astype(np.int64)
    offsets = np.zeros(count, np.int64)
    if count > 1:
        offsets[1:] = np.cumsum(sizes[:-1] + gap)
    total = int(offsets[-1] + sizes[-1])
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    return offsets, sizes, x


def check_against_oracle(offsets, sizes, x, y, sign, every=1):
    for i in range(0, len(sizes), every):
        o, n = int(offsets[i]), int(sizes[i])
        ref = oracle.fft(x[o:o + n][None, :], sign)
        e = oracle.rel_l2(y[o:o + n][None, :], ref)[0]
        assert e < tol(n), (i, n, e)


def emu_packed(emu, offsets, sizes, x, persistent, sign):
    y = np.full_like(x, np.nan + 1j * np.nan)
    err = ctypes.create_string_buffer(512)
    rc = emu.emu_packed_run(offsets.ctypes.data, sizes.ctypes.data, len(sizes), int(persistent), sign,
                            x.ctypes.data, y.ctypes.data, err, len(err))
    return rc, err.value.decode(), y


@pytest.mark.parametrize("persistent", [1, 0])
def test_emulated_mixed_sizes(emu, persistent):
    offsets, sizes, x = make_batch(40, 1, 15, 11, gap=3)
    for sign in (-1, +1):
        rc, msg, y = emu_packed(emu, offsets, sizes, x, persistent, sign)
        assert rc == 0, msg
        check_against_oracle(offsets, sizes, x, y, sign)


def test_emulated_largest_classes(emu):
    offsets = np.array([0, 1 << 16, (1 << 16) + (1 << 17)], np.int64)
    sizes = np.array([1 << 16, 1 << 17, 1 << 18], np.int64)
    rng = np.random.default_rng(5)
    total = int(offsets[-1] + sizes[-1])
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    rc, msg, y = emu_packed(emu, offsets, sizes, x, 1, -1)
    assert rc == 0, msg
    check_against_oracle(offsets, sizes, x, y, -1)


def test_layout_validation(emu):
    x = np.zeros(64, np.complex64)
    bad = [
        (np.array([0, 8], np.int64), np.array([16, 16], np.int64)),   # overlap
        (np.array([0], np.int64), np.array([12], np.int64)),          # not a power of two
        (np.array([0], np.int64), np.array([1 << 19], np.int64)),     # too long
        (np.array([-4], np.int64), np.array([4], np.int64)),          # negative offset
        (np.array([(1 << 62)], np.int64), np.array([4], np.int64)),   # offset beyond 2^40
    ]
    for off, sz in bad:
        rc, msg, _ = emu_packed(emu, off, sz, x, 1, -1)
        assert rc == 2 and msg


def test_emulated_dependency_wait_gives_up(emu):
    """A row item whose column items never run (their launch left out): the
    bounded dependency wait runs out, sets the error word (status 4) and the
    item is skipped, so the output stays untouched; with the column launch
    the same transform completes and agrees with the oracle."""
    offsets, sizes, x = make_batch(1, 13, 13, 21)
    y = np.full_like(x, np.nan + 1j * np.nan)
    err = ctypes.create_string_buffer(512)
    rc = emu.emu_packed_run_launches(offsets.ctypes.data, sizes.ctypes.data, 1, 0, -1, x.ctypes.data, y.ctypes.data,
                                     1, err, len(err))
    assert rc == 4 and "gave up" in err.value.decode()
    assert np.all(np.isnan(y.real))
    rc, msg, y = emu_packed(emu, offsets, sizes, x, False, -1)
    assert rc == 0, msg
    check_against_oracle(offsets, sizes, x, y, -1)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def gpu_packed(offsets, sizes, x_dev, mode, direction):
    import torch

    from estl_gb300._lib import check, lib
    L = lib()
    plan = ctypes.c_void_p()
    check(L.estl_packed_plan_create(offsets.ctypes.data, sizes.ctypes.data, len(sizes), direction, mode,
                                    ctypes.byref(plan)))
    y = torch.full_like(x_dev, float("nan"))
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # graph capture, then replay
        check(L.estl_packed_execute(plan, ctypes.c_void_p(x_dev.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                    ctypes.c_void_p(st)))
    check(L.estl_packed_check(plan))
    buf = ctypes.create_string_buffer(8192)
    check(L.estl_packed_plan_describe(plan, buf, len(buf)))
    desc = json.loads(buf.value.decode())
    L.estl_packed_plan_destroy(plan)
    return y.cpu().numpy(), desc


@pytest.mark.gpu
def test_gpu_uneven_configuration(engine):
    """8192 transforms, log-uniform 2^6..2^16, N(0,1), seed 3: both modes agree
    with each other bit for bit and with the oracle (every 8th transform)."""
    import torch
    offsets, sizes, x = make_batch(8192, 6, 16, 3)
    xd = torch.from_numpy(x).cuda()
    yp, dp = gpu_packed(offsets, sizes, xd, 0, -1)
    ys, ds = gpu_packed(offsets, sizes, xd, 1, -1)
    assert dp["persistent"] and dp["launches"] == 1 and not ds["persistent"] and ds["launches"] >= 11
    assert np.array_equal(yp, ys)
    check_against_oracle(offsets, sizes, x, yp, -1, every=8)


@pytest.mark.gpu
def test_gpu_packed_backward_and_gaps(engine):
    import torch
    offsets, sizes, x = make_batch(300, 1, 18, 7, gap=5)
    xd = torch.from_numpy(x).cuda()
    y, _ = gpu_packed(offsets, sizes, xd, 0, +1)
    check_against_oracle(offsets, sizes, x, y, +1)
    # the gaps between transforms are not written
    mask = np.ones(len(x), bool)
    for o, n in zip(offsets, sizes):
        mask[o:o + n] = False
    assert np.all(np.isnan(y[mask].real))


@pytest.mark.gpu
def test_gpu_execute_packed_one_call(engine):
    """estl_execute_packed (plan, execute, wait, check, release in one call)
    gives the persistent plan's result bit for bit."""
    import torch

    from estl_gb300._lib import check, lib
    offsets, sizes, x = make_batch(500, 3, 15, 11, gap=3)
    xd = torch.from_numpy(x).cuda()
    ref, _ = gpu_packed(offsets, sizes, xd, 0, -1)
    y = torch.full_like(xd, float("nan"))
    check(lib().estl_execute_packed(offsets.ctypes.data, sizes.ctypes.data, len(sizes), -1,
                                    ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    y = y.cpu().numpy()
    mask = np.zeros(len(x), bool)
    for o, n in zip(offsets, sizes):
        mask[o:o + n] = True
    assert np.array_equal(y[mask], ref[mask])
    check_against_oracle(offsets, sizes, x, y, -1, every=10)



@pytest.mark.gpu
def test_gpu_python_packed_api(engine):
    """PackedPlan and fft_packed (the package's wrappers of the packed entry
    points) give the raw C-ABI result bit for bit."""
    import torch
    offsets, sizes, x = make_batch(200, 2, 14, 13, gap=2)
    xd = torch.from_numpy(x).cuda()
    ref, _ = gpu_packed(offsets, sizes, xd, 0, +1)
    p = engine.PackedPlan(offsets, sizes, engine.BACKWARD)
    y = p.execute(xd, out=torch.full_like(xd, float("nan")))
    p.check()
    assert p.describe()["persistent"]
    p.close()
    z = engine.fft_packed(xd, offsets, sizes, inverse=True, out=torch.full_like(xd, float("nan")))
    mask = np.zeros(len(x), bool)
    for o, n in zip(offsets, sizes):
        mask[o:o + n] = True
    assert np.array_equal(y.cpu().numpy()[mask], ref[mask])
    assert np.array_equal(z.cpu().numpy()[mask], ref[mask])


@pytest.mark.gpu
def test_gpu_dependency_wait_gives_up_and_plan_recovers(engine):
    """The bounded dependency wait of the persistent kernel, run out on the
    GPU without a fault: the test hook leaves the four-step column items out
    and bounds the row items' wait at 2^10 polls.  estl_packed_check reports
    ESTL_TIMEOUT, the four-step transforms' outputs are untouched (their row
    items gave up and were skipped), the small transforms are right, and with
    the hook cleared the same plan computes every transform again.  The
    reference's counterpart is its error path (uOpenCL.h:21-55)."""
    import torch

    from estl_gb300._lib import check, lib
    L = lib()
    # two 2^13-point four-step transforms among small single-tile ones
    sizes = np.array([1 << 13, 64, 1 << 13, 256, 1024], np.int64)
    offsets = np.concatenate([[0], np.cumsum(sizes[:-1])]).astype(np.int64)
    rng = np.random.default_rng(21)
    total = int(sizes.sum())
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    plan = ctypes.c_void_p()
    check(L.estl_packed_plan_create(offsets.ctypes.data, sizes.ctypes.data, len(sizes), -1, 0, ctypes.byref(plan)))
    st = torch.cuda.current_stream().cuda_stream
    try:
        check(L.estl_packed_plan_set_test_hook(plan, 1, 1 << 10))
        y = torch.full_like(xd, float("nan"))
        check(L.estl_packed_execute(plan, ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                    ctypes.c_void_p(st)))
        assert L.estl_packed_check(plan) == 6  # ESTL_TIMEOUT
        assert b"gave up" in L.estl_last_error()
        yh = y.cpu().numpy()
        for o, n in zip(offsets, sizes):
            if n == 1 << 13:
                assert np.all(np.isnan(yh[o:o + n].real)), "a skipped row item wrote its output"
            else:
                e = oracle.rel_l2(yh[o:o + n][None, :], oracle.fft(x[o:o + n][None, :], -1))[0]
                assert e < tol(n)
        # hook cleared: the plan runs every item again and reports no timeout
        check(L.estl_packed_plan_set_test_hook(plan, 0, 0))
        y2 = torch.full_like(xd, float("nan"))
        check(L.estl_packed_execute(plan, ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(y2.data_ptr()),
                                    ctypes.c_void_p(st)))
        check(L.estl_packed_check(plan))
        check_against_oracle(offsets, sizes, x, y2.cpu().numpy(), -1)
    finally:
        L.estl_packed_plan_destroy(plan)


def test_python_packed_api_validates_before_the_engine():
    """Argument errors are raised on the host, before any engine call."""
    import torch

    import estl_gb300 as estl
    with pytest.raises(estl.EstlError):
        estl.PackedPlan([0, 16], [16])
    with pytest.raises(estl.EstlError):
        estl.PackedPlan([], [])
    with pytest.raises(estl.EstlError):
        estl.PackedPlan([0], [16], mode="bucketed")
    with pytest.raises(estl.EstlError):  # a host tensor
        estl.fft_packed(torch.zeros(16, dtype=torch.complex64), [0], [16])


def emu_bucketed(emu, offsets, sizes, x, sign):
    y = np.full_like(x, np.nan + 1j * np.nan)
    err = ctypes.create_string_buffer(512)
    rc = emu.emu_packed_bucketed_run(offsets.ctypes.data, sizes.ctypes.data, len(sizes), sign, x.ctypes.data,
                                     y.ctypes.data, err, len(err))
    return rc, err.value.decode(), y


def test_emulated_bucketed_mixed_sizes(emu):
    """Bucketed uneven batches (ESTL_PACKED_BUCKETED): every length runs the
    engine's own plan through the transforms' offsets -- single-CTA tiles,
    the resident 2^13 tile, cluster tiles at 2^14 / 2^15, four-step above --
    with gaps between transforms (odd offsets: plain tiles) and without."""
    for gap in (3, 0):
        offsets, sizes, x = make_batch(30, 1, 16, 41 + gap, gap=gap)
        for sign in (-1, +1):
            rc, msg, y = emu_bucketed(emu, offsets, sizes, x, sign)
            assert rc == 0, msg
            check_against_oracle(offsets, sizes, x, y, sign)
            mask = np.ones(len(x), bool)
            for o, n in zip(offsets, sizes):
                mask[o:o + n] = False
            assert np.all(np.isnan(y[mask].real)), "a gap between transforms was written"


@pytest.mark.gpu
@pytest.mark.parametrize("gap", [0, 3])
def test_gpu_bucketed(engine, gap):
    """ESTL_PACKED_BUCKETED on the GPU against the oracle, both directions,
    graph capture then replay; the gaps stay untouched."""
    import torch
    offsets, sizes, x = make_batch(400, 1, 18, 17 + gap, gap=gap)
    xd = torch.from_numpy(x).cuda()
    for direction in (-1, +1):
        y, desc = gpu_packed(offsets, sizes, xd, 2, direction)
        assert desc["mode"] == "bucketed" and desc["transforms"] == len(sizes)
        check_against_oracle(offsets, sizes, x, y, direction)
        mask = np.ones(len(x), bool)
        for o, n in zip(offsets, sizes):
            mask[o:o + n] = False
        assert np.all(np.isnan(y[mask].real))


# ---------------------------------------------------------------------------
# Mixed batches: transforms and FFT convolutions (Convolution.h:95-154 in 1D)
# in one packed plan.  Convolutions of padded length <= 2^12 are work items of
# the packed kernel (signal and filter as the halves of one complex transform,
# spectra split with X_{-k}); longer ones run the convolution engine's launches.
# ---------------------------------------------------------------------------
CONV_TOL = 1e-6


def conv_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.sum((a - b) ** 2) / max(np.sum(b ** 2), 1e-300)))


def make_convs(shapes, seed, flags=0, scales=None):
    """Requests for (L, K) pairs, packed with gaps of one float; filters
    positive in reference-compatible mode (sum(h) away from zero); optional
    per-request (signal, filter) scales."""
    rng = np.random.default_rng(seed)
    compat = bool(flags & 2)
    reqs, sigs, filts = [], [], []
    so = fo = oo = 0
    for i, (L, K) in enumerate(shapes):
        ss, fs = scales[i] if scales else (1.0, 1.0)
        s = (rng.standard_normal(L) * ss).astype(np.float32)
        f = rng.standard_normal(K).astype(np.float32)
        f = ((np.abs(f) + 0.1) if compat else f) * fs
        reqs.append((L, K, so, fo, oo))
        sigs.append(np.append(s, np.float32(np.nan)))
        filts.append(np.append(f.astype(np.float32), np.float32(np.nan)))
        so += L + 1
        fo += K + 1
        oo += (L if compat else L + K - 1) + 1
    return np.array(reqs, np.int64), np.concatenate(sigs), np.concatenate(filts), oo


def conv_reference(s, f, flags):
    if flags & 2:  # Convolution.h:113-148: cyclic kernel shift by (K+1)/2, / sum(h), L samples
        return oracle.conv_compat(s, f, correlate=bool(flags & 1))
    return oracle.conv_fft(s.astype(np.float64), f.astype(np.float64), correlate=bool(flags & 1))


def check_convs(reqs, sig, filt, cout, flags):
    """rel-L2 per request; in reference-compatible mode relative to the whole
    circular result (the FP32 transforms' rounding is relative to it, and
    the L kept samples of a correlation can be its small tail)."""
    for i, (L, K, so, fo, oo) in enumerate(reqs):
        s, f = sig[so:so + L], filt[fo:fo + K]
        ref = conv_reference(s, f, flags)
        got = cout[oo:oo + len(ref)]
        if flags & 2:
            n = 2
            while n < L + K - 1:
                n *= 2
            full = oracle.conv_circular(s, f, n, bool(flags & 1)) / np.sum(f.astype(np.float64))
            err = float(np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(full))
        else:
            err = conv_rel(got, ref)
        assert err < CONV_TOL, (i, L, K, err)
        assert np.isnan(cout[oo + len(ref)]), (i, "wrote past its output")


def emu_mixed(emu, offsets, sizes, x, persistent, sign, reqs, sig, filt, olen, flags):
    y = np.full_like(x, np.nan + 1j * np.nan)
    cout = np.full(olen, np.nan, np.float32)
    err = ctypes.create_string_buffer(512)
    rc = emu.emu_packed_mixed_run(offsets.ctypes.data, sizes.ctypes.data, len(sizes), int(persistent), sign,
                                  x.ctypes.data, y.ctypes.data, reqs.ctypes.data, len(reqs), flags, sig.ctypes.data,
                                  filt.ctypes.data, cout.ctypes.data, err, len(err))
    return rc, err.value.decode(), y, cout


# padded lengths 2^1..2^12 in the kernel, 2^13 and 2^15 through the engine
MIXED_CONV_SHAPES = [(1, 1), (2, 1), (3, 2), (5, 4), (9, 8), (20, 13), (33, 32), (100, 17), (200, 57), (300, 212),
                     (1000, 25), (1500, 549), (3000, 1000), (2048, 2049), (5000, 300), (20000, 100)]


@pytest.mark.parametrize("flags", [0, 1, 2, 3])
@pytest.mark.parametrize("persistent", [1, 0])
def test_emulated_mixed_transforms_and_convolutions(emu, flags, persistent):
    """A mixed batch through the bounds-checked emulator: transforms of 2^1..2^15
    against oracle.fft and convolutions of every in-kernel padded length (and
    two engine ones) against oracle.conv_fft, every flag combination; the
    floats between requests stay untouched."""
    offsets, sizes, x = make_batch(24, 1, 15, 51, gap=3)
    reqs, sig, filt, olen = make_convs(MIXED_CONV_SHAPES, 52 + flags, flags)
    rc, msg, y, cout = emu_mixed(emu, offsets, sizes, x, persistent, -1, reqs, sig, filt, olen, flags)
    assert rc == 0, msg
    check_against_oracle(offsets, sizes, x, y, -1)
    check_convs(reqs, sig, filt, cout, flags)


def test_emulated_mixed_convolutions_only_and_magnitudes(emu):
    """Only convolutions (no transforms), and requests whose signal and filter
    differ by up to 10^9 in scale: the power-of-two balance of the two halves
    keeps every request at the FP32 tolerance."""
    shapes = [(700, 90), (1000, 20), (60, 3), (2000, 2000), (4, 4)]
    scales = [(1e4, 1e-3), (1e-3, 1e2), (1.0, 1e-5), (1e-4, 1e5), (1.0, 1.0)]
    reqs, sig, filt, olen = make_convs(shapes, 61, 0, scales)
    empty = np.zeros(0, np.int64)
    x = np.zeros(1, np.complex64)
    rc, msg, _, cout = emu_mixed(emu, empty, empty, x, 1, -1, reqs, sig, filt, olen, 0)
    assert rc == 0, msg
    check_convs(reqs, sig, filt, cout, 0)


def test_emulated_mixed_validation(emu):
    offsets, sizes, x = make_batch(2, 4, 6, 1)
    empty = np.zeros(0, np.int64)
    for bad in ([(0, 5, 0, 0, 0)], [(5, 5, -1, 0, 0)], [(1 << 22, 2, 0, 0, 0)], [(5, 5, 1 << 62, 0, 0)],
                [(5, 5, 0, 0, (1 << 40) + 1)]):
        reqs = np.array(bad, np.int64)
        sig = np.zeros(8, np.float32)
        rc, msg, _, _ = emu_mixed(emu, offsets, sizes, x, 1, -1, reqs, sig, sig, 16, 0)
        assert rc == 2 and "convolution 0" in msg, (bad, msg)
    rc, msg, _, _ = emu_mixed(emu, empty, empty, x, 1, -1, np.zeros((0, 5), np.int64), x.real, x.real, 1, 0)
    assert rc == 2 and "at least one" in msg
    reqs, sig, filt, olen = make_convs([(10, 3)], 1)
    rc, msg, _, _ = emu_mixed(emu, offsets, sizes, x, 1, -1, reqs, sig, filt, olen, 1 << 8)
    assert rc == 2 and "FP32" in msg


def random_conv_shapes(count, seed, max_log=12, engine=()):
    """(L, K) pairs whose padded lengths cover 2^1..2^max_log, plus the given
    longer ones (run by the convolution engine)."""
    rng = np.random.default_rng(seed)
    shapes = []
    for _ in range(count):
        lg = int(rng.integers(1, max_log + 1))
        total = int(rng.integers((1 << (lg - 1)) + 1, (1 << lg) + 1)) if lg > 1 else 1
        K = int(rng.integers(1, total + 1))
        shapes.append((total - K + 1, K))
    return shapes + list(engine)


@pytest.mark.gpu
@pytest.mark.parametrize("mode,flags", [(0, 0), (0, 3), (1, 1), (1, 2), (2, 0), (2, 3)])
def test_gpu_mixed_transforms_and_convolutions(engine, mode, flags):
    """A mixed batch on the GPU (estl_packed_mixed_plan_create / _execute):
    300 transforms of 2^1..2^16 against oracle.fft and 404 convolutions
    (padded 2^1..2^12 as work items, 2^13..2^17 on the convolution engine)
    against oracle.conv_fft / oracle.conv_compat, every request checked, in
    each execution mode; the gaps between outputs stay untouched; a second
    execute replays the captured graph."""
    import torch
    offsets, sizes, x = make_batch(300, 1, 16, 81 + mode, gap=1)
    shapes = random_conv_shapes(400, 82 + flags, engine=[(5000, 300), (9000, 3000), (30000, 700), (100000, 31)])
    reqs, sig, filt, olen = make_convs(shapes, 83, flags)
    p = engine.PackedPlan(offsets, sizes, -1, ["persistent", "per_size", "bucketed"][mode], convolutions=reqs,
                          conv_flags=flags)
    d = p.describe()
    assert d["convolutions"] == len(reqs)
    if mode != 2:
        assert d["conv_items"] == len(reqs) - 4 and d["conv_engine"] == 4
    xd = torch.from_numpy(x).cuda()
    sd, fd = torch.from_numpy(sig).cuda(), torch.from_numpy(filt).cuda()
    for rep in range(2):
        yd = torch.full_like(xd, float("nan"))
        cd = torch.full((olen,), float("nan"), dtype=torch.float32, device="cuda")
        p.execute_mixed(xd, yd, sd, fd, cd)
        p.check()
    y, cout = yd.cpu().numpy(), cd.cpu().numpy()
    check_against_oracle(offsets, sizes, x, y, -1)
    check_convs(reqs, sig, filt, cout, flags)
    mask = np.ones(len(x), bool)
    for o, n in zip(offsets, sizes):
        mask[o:o + n] = False
    assert np.all(np.isnan(y[mask].real))
    p.close()


@pytest.mark.gpu
def test_gpu_mixed_convolutions_only_and_errors(engine):
    """A plan of convolutions alone (no transform buffers), its describe, and
    the refusals: a mixed plan through estl_packed_execute, NULL or short
    convolution buffers (before any launch), split precision."""
    import torch
    reqs, sig, filt, olen = make_convs(random_conv_shapes(50, 91, engine=[(20000, 300)]), 92)
    p = engine.PackedPlan([], [], -1, "persistent", convolutions=reqs)
    # the last request ends one float before the end of each array
    assert p.conv_extents == (sig.size - 1, filt.size - 1, olen - 1)
    sd, fd = torch.from_numpy(sig).cuda(), torch.from_numpy(filt).cuda()
    cd = torch.full((olen,), float("nan"), dtype=torch.float32, device="cuda")
    p.execute_mixed(None, None, sd, fd, cd)
    p.check()
    check_convs(reqs, sig, filt, cd.cpu().numpy(), 0)
    with pytest.raises(engine.EstlError):
        p.execute(torch.zeros(4, dtype=torch.complex64, device="cuda"))
    with pytest.raises(engine.EstlError):
        p.execute_mixed(None, None, sd, fd, None)
    for short in ((sd[:-2], fd, cd), (sd, fd[:-2], cd), (sd, fd, cd[:-2])):
        with pytest.raises(engine.EstlError):
            p.execute_mixed(None, None, *short)
    p.close()
    b = engine.PackedPlan([], [], -1, "bucketed", convolutions=reqs)
    assert b.conv_extents == (sig.size - 1, filt.size - 1, olen - 1)
    b.close()
    with pytest.raises(engine.EstlError):
        engine.PackedPlan([], [], -1, "persistent", convolutions=reqs, conv_flags=1 << 8)
