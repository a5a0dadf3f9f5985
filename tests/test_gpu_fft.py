"""GPU parity of the batched C2C FP32 FFT against the FP64 oracle, through the
C ABI (libestl_cuda.so via ctypes).

Tolerances (relative L2 per transform, the metric of OpenCL_FFT/main.cpp:333-359
without the division by FLT_EPSILON): 2e-6 for N <= 2^20 and
c * log2(N) * 2^-24 with c = 2 beyond.
"""
import ctypes
import math

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def tol(n):
    return 2e-6 if n <= (1 << 20) else 2.0 * math.log2(n) * 2.0 ** -24


def uniform_c64(shape, seed):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64)


def run(engine, x_np, direction):
    import torch
    batch, n = x_np.shape
    p = engine.Plan(n, batch, direction)
    xd = torch.from_numpy(x_np).cuda()
    yd = p.execute(xd)
    torch.cuda.synchronize()
    return yd.cpu().numpy(), p


@pytest.mark.parametrize("logn", range(0, 25))
def test_parity_every_size(engine, logn):
    n = 1 << logn
    batch = max(1, min(5, (1 << 22) // n))
    x = uniform_c64((batch, n), 1000 + logn)
    for direction in (-1, +1):
        y, _ = run(engine, x, direction)
        e = oracle.rel_l2(y, oracle.fft(x, direction))
        assert e.max() < tol(n), (n, direction, e.max())


def test_config1_plain_4096x256(engine):
    """N = 4096, batch = 256, uniform[-1,1) seed 1: every transform vs the oracle."""
    x = uniform_c64((256, 4096), 1)
    y, p = run(engine, x, -1)
    e = oracle.rel_l2(y, oracle.fft(x, -1))
    assert e.max() < 2e-6
    assert p.describe()["hbm_passes"] == 1


def test_known_answer_like_reference(engine):
    """tests/Test.cpp:60-77 through the engine: cosine -> spikes of M/2."""
    for m in (4, 10, 12, 16):
        M = 1 << m
        B = 8
        q = np.arange(M)
        x = np.empty((B, M), np.complex64)
        expect = np.zeros((B, M), np.complex128)
        for b in range(B):
            eff = ((1 + b) % (M // 2 - 1)) + 1
            x[b] = np.cos(2 * np.pi * (eff * q) / M).astype(np.float32)
            expect[b, eff] += M / 2
            expect[b, M - eff] += M / 2
        y, _ = run(engine, x, -1)
        assert (np.abs(y - expect) ** 2).max() < 1e-3 * M


@pytest.mark.parametrize("logn", [10, 12, 14, 16, 20, 24])
def test_full_size_sweep_properties(engine, logn):
    """Sweep configuration (N * batch = 2^27, 1 GiB): round trip, Parseval and
    oracle spot checks of the first and last transform."""
    import torch
    n = 1 << logn
    batch = (1 << 27) // n
    g = torch.Generator(device="cuda").manual_seed(2)
    x = (torch.rand((batch, n, 2), device="cuda", generator=g) * 2 - 1).contiguous()
    xc = torch.view_as_complex(x)
    fwd = engine.Plan(n, batch, -1)
    bwd = engine.Plan(n, batch, +1)
    y = fwd.execute(xc)
    z = bwd.execute(y)
    torch.cuda.synchronize()
    rt = ((z / n - xc).abs().double() ** 2).sum(-1).sqrt() / (xc.abs().double() ** 2).sum(-1).sqrt()
    assert rt.max().item() < 2 * tol(n)
    px = (xc.abs().double() ** 2).sum(-1) * n
    py = (y.abs().double() ** 2).sum(-1)
    assert ((py - px).abs() / px).max().item() < 1e-5
    for b in (0, batch - 1):
        xb = xc[b].cpu().numpy()[None, :]
        assert oracle.rel_l2(y[b].cpu().numpy()[None, :], oracle.fft(xb, -1)).max() < tol(n)
    del x, xc, y, z


def test_execute_host_matches_device(engine):
    import torch
    for n, batch in ((4096, 64), (1 << 16, 40), (1 << 20, 3)):
        x = uniform_c64((batch, n), n)
        p = engine.Plan(n, batch, -1)
        yd = p.execute(torch.from_numpy(x).cuda()).cpu().numpy()
        xh = torch.from_numpy(x).pin_memory().numpy()
        yh = torch.empty((batch, n), dtype=torch.complex64).pin_memory().numpy()
        p.execute_host(xh, yh)
        assert np.array_equal(yh, yd)
        yp = np.zeros_like(x)  # pageable output
        p.execute_host(x, yp)
        assert np.array_equal(yp, yd)


def sentinel_c64(count, device="cuda"):
    """count complex64 elements, every one 1234.5 - 6789.25i."""
    import torch
    g = torch.empty((count, 2), dtype=torch.float32, device=device)
    g[:, 0] = 1234.5
    g[:, 1] = -6789.25
    return torch.view_as_complex(g)


@pytest.mark.parametrize("logn", range(1, 9))
def test_small_sizes_every_batch_with_guards(engine, logn):
    """N = 2..2^8, every batch 1..17, both directions: results against the
    oracle, the input unchanged, and guard regions of sentinel values on both
    sides of the input and of the output untouched (nothing written outside
    the output)."""
    import torch
    n = 1 << logn
    G = 1024  # guard elements on each side (8 KiB: keeps both buffers 16-byte aligned)
    s = complex(1234.5, -6789.25)
    st = torch.cuda.current_stream().cuda_stream
    for batch in range(1, 18):
        m = batch * n
        x = uniform_c64((batch, n), 5000 + 100 * logn + batch)
        xin = sentinel_c64(m + 2 * G)
        xin[G:G + m] = torch.from_numpy(x.reshape(-1)).cuda()
        for direction in (-1, +1):
            out = sentinel_c64(m + 2 * G)
            p = engine.Plan(n, batch, direction)
            p.execute_ptr(xin.data_ptr() + 8 * G, out.data_ptr() + 8 * G, st)
            torch.cuda.synchronize()
            o = out.cpu().numpy()
            xi = xin.cpu().numpy()
            assert np.all(o[:G] == s) and np.all(o[G + m:] == s), (n, batch, direction)
            assert np.all(xi[:G] == s) and np.all(xi[G + m:] == s) and np.array_equal(xi[G:G + m], x.reshape(-1))
            e = oracle.rel_l2(o[G:G + m].reshape(batch, n), oracle.fft(x, direction))
            assert e.max() < tol(n), (n, batch, direction, e.max())
            p.close()


def test_non_default_stream(engine):
    import torch
    x = uniform_c64((16, 1 << 15), 3)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        xd = torch.from_numpy(x).cuda()
        p = engine.Plan(1 << 15, 16, -1)
        yd = p.execute(xd, stream=s)
    s.synchronize()
    assert oracle.rel_l2(yd.cpu().numpy(), oracle.fft(x, -1)).max() < 2e-6


def test_errors(engine):
    import torch
    from estl_gb300 import EstlError
    with pytest.raises(EstlError) as e:
        engine.Plan((1 << 23) + 3, 1)  # beyond the Bluestein limit for other lengths
    assert e.value.name == "ESTL_UNSUPPORTED_SIZE"
    with pytest.raises(EstlError) as e:
        engine.Plan(1 << 25, 1)
    assert e.value.name == "ESTL_UNSUPPORTED_SIZE"
    with pytest.raises(EstlError) as e:
        engine.Plan(16, 0)
    assert e.value.name == "ESTL_INVALID_ARG"
    p = engine.Plan(16, 4)
    x = torch.zeros(64, dtype=torch.complex64, device="cuda")
    with pytest.raises(EstlError):
        p.execute_ptr(x.data_ptr(), x.data_ptr())  # in-place
    with pytest.raises(EstlError):
        p.execute_ptr(x.data_ptr() + 4, x.data_ptr() + 256)  # misaligned
    assert engine.max_batch(4096) > 1000
    # Bluestein lengths: the budget less the plan's fixed buffers; out-of-range lengths: 0
    assert engine.max_batch(1000) > 1000 and engine.max_batch(1 << 23) > 0
    assert engine.max_batch(1 << 25) == 0 and engine.max_batch((1 << 23) + 1) == 0 and engine.max_batch(0) == 0


def test_hbm_budget_refusal_leaves_nothing_behind(engine):
    """Allocator failure made on the host: with the budget 1 MiB above the
    bytes in use, plans that need device scratch (four-step 2^20, Bluestein
    10^6) are refused with ESTL_OUT_OF_MEMORY and the bytes in use do not
    change; a single-pass plan, which needs none, still runs; the budget is
    restored afterwards."""
    from estl_gb300 import EstlError
    used, budget = engine.memory_usage()
    try:
        engine.init(0, used + (1 << 20))
        for n, batch in ((1 << 20, 16), (1000000, 4)):
            with pytest.raises(EstlError) as e:
                engine.Plan(n, batch, -1)
            assert e.value.name == "ESTL_OUT_OF_MEMORY", (n, str(e.value))
            assert engine.memory_usage()[0] == used
        x = uniform_c64((4, 4096), 9)
        y, p = run(engine, x, -1)
        assert oracle.rel_l2(y, oracle.fft(x, -1)).max() < 2e-6
        p.close()
    finally:
        engine.init(0, budget)
    assert engine.memory_usage()[1] == budget


def test_autotune_keeps_results(engine, tmp_path, monkeypatch):
    import torch
    monkeypatch.setenv("ESTL_TUNE_CACHE", str(tmp_path / "tune.jsonl"))
    n, batch = 1 << 16, 64
    res = engine.autotune(n, batch, iters=3)
    assert res["candidates"] > 1 and res["best_ms"] > 0
    assert (tmp_path / "tune.jsonl").exists()
    x = uniform_c64((batch, n), 5)
    y = engine.Plan(n, batch, -1).execute(torch.from_numpy(x).cuda()).cpu().numpy()
    assert oracle.rel_l2(y, oracle.fft(x, -1)).max() < 2e-6


@pytest.mark.parametrize("logn,split,row_e,row_c", [(16, 8, 4, 3), (18, 9, 4, 2), (19, 9, 4, 2), (20, 10, 4, 2),
                                                    (21, 10, 4, 1), (22, 11, 4, 2), (23, 11, 4, 1), (24, 12, 4, 1)])
def test_bulk_load_row_tiles(engine, logn, split, row_e, row_c):
    """The persistent row pass with bulk asynchronous tile loads (pipelined = 2,
    bulk_core.cuh) against the oracle, both directions, and its wait-timeout
    word clear afterwards."""
    import torch
    n = 1 << logn
    batch = max(2, (1 << 23) // n)
    x = uniform_c64((batch, n), 700 + logn)
    xd = torch.from_numpy(x).cuda()
    row_m = logn - split
    for direction in (-1, +1):
        p = engine.Plan(n, batch, direction, mode="four_step",
                        tiles={"split_log2": split, "row_loge": row_e, "row_logc": row_c, "pipelined": 2})
        d = p.describe()
        assert d["kernels"][1]["kind"] == "row" and d["kernels"][1]["pipe"] == 2 and d["kernels"][1]["logm"] == row_m
        y = p.execute(xd)
        p.check()
        assert oracle.rel_l2(y.cpu().numpy(), oracle.fft(x, direction)).max() < tol(n)


@pytest.mark.parametrize("logn,col", [(16, (7, 4, 5)), (17, (8, 4, 4)), (17, (8, 4, 3)), (18, (9, 4, 3)),
                                      (20, (9, 4, 4)), (19, (10, 4, 2)), (21, (10, 4, 3)), (22, (11, 4, 2)),
                                      (24, (12, 4, 1))])
def test_tensor_copy_column_tiles(engine, logn, col):
    """The persistent column pass whose strided tiles arrive as 2D tensor
    copies (pipelined = 2, bulk_core.cuh BulkColKernel) against the oracle,
    both directions, and its wait-timeout word clear afterwards."""
    import torch
    logm, loge, logc = col
    n = 1 << logn
    batch = max(2, (1 << 23) // n)
    x = uniform_c64((batch, n), 800 + logn)
    xd = torch.from_numpy(x).cuda()
    for direction in (-1, +1):
        p = engine.Plan(n, batch, direction, mode="four_step",
                        tiles={"split_log2": logm, "col_loge": loge, "col_logc": logc, "row_loge": 4, "row_logc": 2,
                               "pipelined": 2})
        d = p.describe()
        assert d["kernels"][0]["kind"] == "col" and d["kernels"][0]["pipe"] == 2 and d["kernels"][0]["logm"] == logm
        y = p.execute(xd)
        p.check()
        assert oracle.rel_l2(y.cpu().numpy(), oracle.fft(x, direction)).max() < tol(n)


@pytest.mark.parametrize("logn,lr,lq,pipe", [(21, 7, 7, 2), (22, 8, 7, 0), (23, 8, 8, 2), (23, 8, 7, 2),
                                             (24, 8, 8, 0), (24, 8, 8, 2), (24, 9, 8, 2)])
def test_three_pass(engine, logn, lr, lq, pipe):
    """Three-pass plans (mode three_pass: column DFTs of 2^lr, column DFTs of
    2^lq stored as interleaved rows, row DFTs) against the oracle, both
    directions, with two transforms per launch."""
    import torch
    n = 1 << logn
    x = uniform_c64((2, n), 900 + logn)
    xd = torch.from_numpy(x).cuda()
    for direction in (-1, +1):
        p = engine.Plan(n, 2, direction, mode="three_pass", tiles={"split_log2": lr, "split2_log2": lq, "pipelined": pipe})
        d = p.describe()
        assert d["hbm_passes"] == 3 and [k["logm"] for k in d["kernels"]] == [lr, lq, logn - lr - lq]
        y = p.execute(xd)
        p.check()
        assert oracle.rel_l2(y.cpu().numpy(), oracle.fft(x, direction)).max() < tol(n)


@pytest.mark.parametrize("logn", range(9, 15))
def test_radix32_single_tiles(engine, logn):
    """Single-tile kernels with radix-32 passes (32 elements per thread)
    against the oracle, both directions."""
    import torch
    n = 1 << logn
    logc = {9: 4, 10: 3, 11: 2, 12: 1, 13: 0, 14: 0}[logn]
    x = uniform_c64((max(3, (1 << 20) // n), n), 1100 + logn)
    xd = torch.from_numpy(x).cuda()
    for direction in (-1, +1):
        p = engine.Plan(n, x.shape[0], direction, mode="single",
                        tiles={"single_loge": 5, "single_logc": logc, "single_logr": 5})
        y = p.execute(xd).cpu().numpy()
        assert oracle.rel_l2(y, oracle.fft(x, direction)).max() < tol(n)


@pytest.mark.parametrize("logn,split,col,row,pipe", [(18, 9, (5, 3), (5, 3), 0), (19, 9, (5, 4), (5, 2), 2),
                                                     (19, 10, (5, 3), (5, 3), 2), (20, 10, (5, 2), (5, 2), 2),
                                                     (20, 10, (5, 3), (5, 2), 0), (21, 10, (5, 3), (4, 2), 2)])
def test_radix32_four_step_tiles(engine, logn, split, col, row, pipe):
    """Four-step column / row tiles with radix-32 passes, plain and bulk-load."""
    import torch
    n = 1 << logn
    x = uniform_c64((2, n), 1200 + logn)
    xd = torch.from_numpy(x).cuda()
    tiles = {"split_log2": split, "col_loge": col[0], "col_logc": col[1], "col_logr": 5,
             "row_loge": row[0], "row_logc": row[1], "row_logr": 5 if row[0] == 5 else -1, "pipelined": pipe}
    for direction in (-1, +1):
        p = engine.Plan(n, 2, direction, mode="four_step", tiles=tiles)
        y = p.execute(xd)
        p.check()
        assert oracle.rel_l2(y.cpu().numpy(), oracle.fft(x, direction)).max() < tol(n)


@pytest.mark.parametrize("logn,logr", [(12, 4), (13, 4), (13, 5)])
def test_bulk_single_tiles(engine, logn, logr):
    """Single-tile sizes on the persistent bulk-load row tile (one whole
    transform per tile), both directions, against the oracle."""
    import torch
    n = 1 << logn
    x = uniform_c64(((1 << 22) // n, n), 1300 + logn)
    xd = torch.from_numpy(x).cuda()
    for direction in (-1, +1):
        p = engine.Plan(n, x.shape[0], direction, mode="single",
                        tiles={"single_loge": 5, "single_logc": 0, "single_logr": logr, "pipelined": 2})
        d = p.describe()
        assert d["kernels"][0]["kind"] == "row" and d["kernels"][0]["pipe"] == 2
        y = p.execute(xd)
        p.check()
        assert oracle.rel_l2(y.cpu().numpy(), oracle.fft(x, direction)).max() < tol(n)


@pytest.mark.parametrize("logn,loge,logr,rounds", [(12, 4, 4, 1), (13, 4, 4, 1), (13, 4, 4, 2), (13, 5, 5, 1),
                                                   (13, 5, 5, 2), (14, 4, 4, 2), (14, 5, 5, 2), (14, 5, 4, 2)])
def test_resident_single_tiles(engine, logn, loge, logr, rounds):
    """Whole transforms on the persistent resident tiles (resident_core.cuh:
    the next transform's bulk copy overlaps this one's passes; exchanges in a
    whole or half tile), both directions, against the oracle.  The batch is
    not a multiple of the grid, so CTAs run different tile counts."""
    import torch
    n = 1 << logn
    x = uniform_c64(((1 << 23) // n + 3, n), 1400 + logn + 10 * rounds)
    xd = torch.from_numpy(x).cuda()
    for direction in (-1, +1):
        p = engine.Plan(n, x.shape[0], direction, mode="single",
                        tiles={"single_loge": loge, "single_logc": 0, "single_logr": logr, "pipelined": 2 + rounds})
        d = p.describe()
        assert d["kernels"][0]["kind"] == "single" and d["kernels"][0]["pipe"] == 2 + rounds
        y = p.execute(xd)
        p.check()
        assert oracle.rel_l2(y.cpu().numpy(), oracle.fft(x, direction)).max() < tol(n)


CLUSTER_TILES = [(12, 1, 6, 4), (12, 2, 6, 4), (13, 1, 7, 4), (14, 1, 7, 4), (14, 2, 7, 4), (14, 1, 7, 5), (15, 2, 7, 4), (15, 2, 8, 4),
                 (15, 3, 8, 4), (15, 2, 8, 5), (16, 3, 7, 4), (16, 3, 8, 4), (16, 3, 8, 5), (16, 4, 8, 4), (17, 4, 8, 4),
                 (17, 4, 9, 4)]


@pytest.mark.parametrize("logn,lcl,logn2,loge", CLUSTER_TILES)
def test_cluster_tiles(engine, logn, lcl, logn2, loge):
    """One transform per thread-block cluster of 2^lcl CTAs (cluster_core.cuh:
    column DFTs, the four-step transpose through distributed shared memory,
    row DFTs; one HBM pass), both directions, against the oracle."""
    import torch
    n = 1 << logn
    x = uniform_c64(((1 << 23) // n + 1, n), 1500 + logn + lcl)
    xd = torch.from_numpy(x).cuda()
    for direction in (-1, +1):
        p = engine.Plan(n, x.shape[0], direction, mode="single",
                        tiles={"single_loge": loge, "single_cluster_log2": lcl, "split_log2": logn2})
        d = p.describe()
        assert d["hbm_passes"] == 1 and d["kernels"][0]["cluster"] == lcl
        y = p.execute(xd)
        p.check()
        assert oracle.rel_l2(y.cpu().numpy(), oracle.fft(x, direction)).max() < tol(n)


@pytest.mark.parametrize("n,batch", [(4096, 4 * 2048 + 5), (1 << 18, 4 * 32 + 7), (1 << 13, 4 * 1024)])
def test_execute_host_ramped_chunks(engine, n, batch):
    """Host pipelines long enough for the opening and closing ramp of smaller
    chunks (1/8, 1/4, 1/2 of the 64 MiB chunk): bit-identical to the device
    execute, forward and backward."""
    import torch
    rng = np.random.default_rng(n + batch)
    x = rng.standard_normal((batch, n, 2), dtype=np.float32).view(np.complex64)[..., 0]
    xh = torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
    yh = torch.empty_like(xh).pin_memory()
    xd = xh.cuda()
    for direction in (-1, +1):
        p = engine.Plan(n, batch, direction)
        yd = p.execute(xd).cpu()
        p.execute_host(xh.numpy(), yh.numpy())
        assert torch.equal(yh, yd)
        p.close()
