"""Every tile kernel configuration and every plan shape, run through the host
emulator (tests/emu/emu.cpp): the kernel bodies of estl_gb300/csrc/fft_core.cuh
with bounds-checked global/shared/twiddle accesses and real barriers.

This is the pre-flight check for GPU launches: a configuration that reads or
writes outside its buffers, or reads shared memory it never wrote, fails here
on the CPU (poisoned shared memory shows up as NaN in the output).
"""
import ctypes
import json

import numpy as np
import pytest

import oracle

TOL = 2e-6  # rel-L2 bound for FP32 results, N <= 2^20


def rand_c64(shape, seed):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64)


def pad_choice(choice):
    """PlanChoice fields: mode, single_loge, single_logc, logn2, col_loge,
    col_logc, row_loge, row_logc, chunk, lag, pipe (0 plain, 2 bulk-load, 3 / 4 resident),
    split (0 FP32, 1 fp16x2, 2 bf16x2, 3 bf16x3 tensor-core radix-16 passes),
    logn3 (three-pass: log2 of the second column DFT length, 0 = default),
    single_logr, col_logr, row_logr (log2 largest radix, -1 = 16),
    single_cluster (log2 CTAs per transform of a cluster tile, -1 = default)."""
    c = list(choice)
    if len(c) < 13:
        c += [0] * (13 - len(c))
    if len(c) < 17:
        c += [-1] * (17 - len(c))
    return c


def emu_run(emu, n, batch, x, sign=-1, choice=None):
    y = np.full((batch, n), np.nan + 1j * np.nan, dtype=np.complex64)
    err = ctypes.create_string_buffer(512)
    ch = None
    if choice is not None:
        ch = (ctypes.c_int * 17)(*pad_choice(choice))
    rc = emu.emu_plan_run(n, batch, ch, sign, x.ctypes.data, y.ctypes.data, err, len(err))
    return rc, err.value.decode(), y


def candidates(emu, n, batch):
    buf = (ctypes.c_int * (17 * 4096))()
    k = emu.emu_plan_candidates(n, batch, buf, 4096)
    return [list(buf[17 * i: 17 * i + 17]) for i in range(min(k, 4096))]


def describe(emu, n, batch, choice=None):
    buf = ctypes.create_string_buffer(2048)
    ch = (ctypes.c_int * 17)(*pad_choice(choice)) if choice is not None else None
    rc = emu.emu_plan_describe(n, batch, ch, buf, len(buf))
    assert rc == 0, buf.value
    return json.loads(buf.value.decode())


@pytest.mark.parametrize("logn", range(0, 15))
def test_default_plans_small(emu, logn):
    n = 1 << logn
    for batch in (1, 3):
        x = rand_c64((batch, n), logn * 10 + batch)
        for sign in (-1, +1):
            rc, msg, y = emu_run(emu, n, batch, x, sign)
            assert rc == 0, msg
            assert np.all(np.isfinite(y))
            assert oracle.rel_l2(y, oracle.fft(x, sign)).max() < TOL


@pytest.mark.parametrize("logn", range(1, 15))
def test_every_single_kernel_config(emu, logn):
    """All instantiated single-kernel tiles, with a ragged last CTA."""
    n = 1 << logn
    cands = [c for c in candidates(emu, n, 5) if c[0] == 1]
    assert cands, "no single-kernel candidates"
    for c in cands:
        per_cta = 1 << c[2]
        batch = per_cta + 1 if per_cta < 64 else 3
        x = rand_c64((batch, n), 7 + logn)
        rc, msg, y = emu_run(emu, n, batch, x, -1, c)
        assert rc == 0, (c, msg)
        assert oracle.rel_l2(y, oracle.fft(x, -1)).max() < TOL, c


@pytest.mark.parametrize("logn", [14, 16, 19])
def test_every_four_step_config(emu, logn):
    """Every column tile and every row tile the autotuner may pick (each at
    least once, plain and bulk-load), with a chunk of two transforms."""
    n = 1 << logn
    cands = [c for c in candidates(emu, n, 2) if c[0] == 2]
    assert cands
    x = rand_c64((2, n), logn)
    ref = oracle.fft(x, +1)
    seen_col, seen_row = set(), set()
    for c in cands:
        col = (c[3], c[4], c[5], c[10])
        row = (c[3], c[6], c[7], c[10])
        if col in seen_col and row in seen_row:
            continue
        seen_col.add(col)
        seen_row.add(row)
        c = list(c)
        c[8] = 1  # one transform per chunk: exercises the chunk loop
        rc, msg, y = emu_run(emu, n, 2, x, +1, c)
        assert rc == 0, (c, msg)
        assert oracle.rel_l2(y, ref).max() < TOL, c


@pytest.mark.parametrize("logn", [18, 20])
def test_four_step_large(emu, logn):
    n = 1 << logn
    x = rand_c64((1, n), logn)
    rc, msg, y = emu_run(emu, n, 1, x, -1)
    assert rc == 0, msg
    assert oracle.rel_l2(y, oracle.fft(x, -1)).max() < TOL


def test_plan_shapes(emu):
    assert describe(emu, 1, 7)["kernels"][0]["kind"] == "copy"
    d = describe(emu, 4096, 256)
    assert d["hbm_passes"] == 1 and d["launches"] == 1 and d["kernels"][0]["kind"] == "single"
    d = describe(emu, 1 << 20, 128)
    assert d["hbm_passes"] == 2 and d["kernels"][0]["kind"] == "col" and d["kernels"][1]["kind"] == "row"
    assert d["scratch_bytes"] <= 1 << 30
    d = describe(emu, 1 << 24, 16)
    assert d["launches"] == 6  # 1 GiB scratch = eight 2^24-point transforms per chunk, 3 launches per chunk
    # the default of 2^24: three passes, 2^7 x 2^8 column DFTs and 2^9-point rows, bulk-load tiles
    assert d["hbm_passes"] == 3
    assert [(k["kind"], k["logm"], k["pipe"]) for k in d["kernels"]] == [("col", 7, 2), ("col", 8, 2), ("row", 9, 2)]
    d = describe(emu, 1 << 24, 16, [2, -1, -1, -1, -1, -1, -1, -1])
    # the tuned four-step of 2^24: 2^12 x 2^12 with 32-element column and row tiles of 4 columns / rows
    assert [(k["logm"], k["loge"], k["logc"]) for k in d["kernels"]] == [(12, 5, 2), (12, 5, 2)]


def test_rejects_bad_sizes(emu):
    x = np.zeros((1, 16), np.complex64)
    for n in (3, 12, 1 << 25, 0):
        rc, msg, _ = emu_run(emu, n, 1, np.zeros((1, max(n, 1)), np.complex64))
        assert rc == 2 and msg
    rc, msg, _ = emu_run(emu, 16, 0, x)
    assert rc == 2


def test_rejects_totals_beyond_2e40(emu):
    """n * batch above 2^40 elements is refused by the planner (no 64-bit
    product of sizes can overflow); exactly 2^40 is planned."""
    buf = ctypes.create_string_buffer(2048)
    assert emu.emu_plan_describe(1 << 24, 1 << 17, None, buf, len(buf)) == 2 and b"2^40" in buf.value
    assert emu.emu_plan_describe(1 << 24, 1 << 16, None, buf, len(buf)) == 0
    assert emu.emu_plan_describe(16, (1 << 62) + 1, None, buf, len(buf)) == 2
    z = np.zeros(4, np.complex64)
    err = ctypes.create_string_buffer(512)
    assert emu.emu_plan2d_run(1 << 10, 1 << 10, 1 << 21, -1, z.ctypes.data, z.ctypes.data, err, len(err)) == 2
    assert emu.emu_bluestein_run(1000, 1 << 31, -1, z.ctypes.data, z.ctypes.data, err, len(err)) == 2
    assert b"2^40" in err.value


def test_twiddle_bank_accuracy(emu):
    """The bank holds w_{2^k}^j rounded once from higher precision."""
    size = emu.emu_bank(None)
    bank = np.empty(size, np.complex64)
    emu.emu_bank(bank.ctypes.data)
    for k in (1, 4, 12, 18):
        j = np.arange(1 << k)
        exact = np.exp(-2j * np.pi * j / (1 << k))
        got = bank[(1 << k) + j]
        assert np.abs(got - exact).max() < 6e-8


@pytest.mark.parametrize("col", [(7, 4, 5), (8, 4, 3), (9, 4, 4), (10, 4, 2), (11, 4, 2), (12, 4, 1)])
def test_tensor_copy_column_tiles(emu, col):
    """The persistent column pass whose tiles arrive as 2D tensor copies
    (bulk_core.cuh BulkColKernel, pipelined = 2): the emulated boxes check the
    16-byte x offset, the 128-byte shared-memory alignment and the source
    bounds of every box; two CTAs loop over the tiles through both stages."""
    logm, loge, logc = col
    logn = logm + 9
    n = 1 << logn
    choice = [2, -1, -1, logm, loge, logc, 4, 2, 0, 0, 2]
    d = describe(emu, n, 2, choice)
    assert d["kernels"][0]["kind"] == "col" and d["kernels"][0]["pipe"] == 2
    x = rand_c64((2, n), 90 + logm)
    for sign in (-1, +1):
        rc, msg, y = emu_run(emu, n, 2, x, sign, choice)
        assert rc == 0, msg
        assert oracle.rel_l2(y, oracle.fft(x, sign)).max() < TOL


@pytest.mark.parametrize("logn,lr,lq,pipe", [(21, 7, 7, 0), (21, 7, 7, 2), (22, 8, 7, 2), (22, 7, 8, 0)])
def test_three_pass(emu, logn, lr, lq, pipe):
    """Three-pass plan (mode 4): column DFTs of 2^lr and 2^lq, the middle
    pass storing interleaved rows, then row DFTs; both directions, plain and
    bulk-load tiles, against the oracle."""
    n = 1 << logn
    choice = [4, -1, -1, lr, -1, -1, -1, -1, 0, 0, pipe, 0, lq]
    d = describe(emu, n, 1, choice)
    assert d["hbm_passes"] == 3 and [k["kind"] for k in d["kernels"]] == ["col", "col", "row"]
    assert [k["logm"] for k in d["kernels"]] == [lr, lq, logn - lr - lq]
    assert all(k["pipe"] == pipe for k in d["kernels"][:2])
    x = rand_c64((1, n), 60 + logn)
    for sign in (-1, +1):
        rc, msg, y = emu_run(emu, n, 1, x, sign, choice)
        assert rc == 0, msg
        assert oracle.rel_l2(y, oracle.fft(x, sign)).max() < 2 * logn * 2.0 ** -24


@pytest.mark.parametrize("logn,loge,logr", [(12, 5, 4), (13, 5, 4), (13, 5, 5)])
def test_bulk_single_tiles(emu, logn, loge, logr):
    """Single-tile sizes on the persistent bulk-load row tile with one whole
    transform per tile (pipelined = 2, N2 = 1), two CTAs looping over five
    transforms through both stages."""
    n = 1 << logn
    choice = [1, loge, 0, -1, -1, -1, -1, -1, 0, 0, 2, 0, 0, logr, -1, -1]
    d = describe(emu, n, 5, choice)
    assert d["kernels"][0]["kind"] == "row" and d["kernels"][0]["pipe"] == 2 and d["hbm_passes"] == 1
    x = rand_c64((5, n), 70 + logn)
    for sign in (-1, +1):
        rc, msg, y = emu_run(emu, n, 5, x, sign, choice)
        assert rc == 0, msg
        assert oracle.rel_l2(y, oracle.fft(x, sign)).max() < TOL


@pytest.mark.parametrize("logn", range(1, 9))
def test_exhaustive_small_sizes_and_batches(emu, logn):
    """Small sizes exhaustively: N = 2..2^8, every batch 1..17 (ragged last
    CTAs of every tile), both directions, default plans, against the oracle."""
    n = 1 << logn
    for batch in range(1, 18):
        x = rand_c64((batch, n), 100 * logn + batch)
        for sign in (-1, +1):
            rc, msg, y = emu_run(emu, n, batch, x, sign)
            assert rc == 0, (n, batch, msg)
            assert oracle.rel_l2(y, oracle.fft(x, sign)).max() < TOL, (n, batch, sign)


def cluster_candidates(emu, n):
    return [c for c in candidates(emu, n, 2) if c[0] == 1 and c[16] > 0]


def test_cluster_scheduler_orders_distributed_shared_memory(emu):
    """The emulated cluster barrier orders another CTA's shared-memory writes
    before this CTA's reads; __syncthreads alone does not (in one of the two
    scheduling orders the neighbour's slot still holds the poison)."""
    for ncta in (2, 4, 8):
        assert emu.emu_cluster_barrier_selftest(ncta, 64, 1) == ncta * 64
        assert emu.emu_cluster_barrier_selftest(ncta, 64, 0) < ncta * 64


@pytest.mark.parametrize("logn", range(12, 18))
def test_cluster_tiles(emu, logn):
    """Every cluster tile (one transform per thread-block cluster, the
    four-step transpose through distributed shared memory), both directions,
    two transforms (two clusters: forward and reverse scheduling order)."""
    n = 1 << logn
    cands = cluster_candidates(emu, n)
    assert cands, "no cluster tiles"
    x = rand_c64((2, n), 50 + logn)
    for c in cands:
        for sign in (-1, +1):
            rc, msg, y = emu_run(emu, n, 2, x, sign, c)
            assert rc == 0, (c, msg)
            assert oracle.rel_l2(y, oracle.fft(x, sign)).max() < (TOL if n <= 1 << 20 else 1e-5), c
        d = describe(emu, n, 2, c)
        assert d["hbm_passes"] == 1 and d["kernels"][0]["cluster"] == c[16]
