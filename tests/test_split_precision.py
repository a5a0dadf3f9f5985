"""Split-precision tensor-core path on the host emulator (tc_core.cuh): the
staging, split, scaling and scatter of every radix-16 pass run through the
emulator's bounds-checked shared memory, with the tensor-core products
computed from the staged 16-bit terms.  Errors are against the FP64 oracle
with 1% of the inputs scaled by 1e3 (the dynamic-range stress of the
split-precision benchmark configuration).

Tolerances (relative L2 per transform): fp16 hi+lo and bf16 hi+mid+lo carry
22-24 significant bits and stay within the 2e-6 FP32 target; bf16 hi+lo
carries 16 bits (about 1e-5 relative per stage)."""
import ctypes

import numpy as np
import pytest

import oracle
from test_emulator import describe, emu_run, rand_c64

TOL = {1: 2e-6, 2: 3e-5, 3: 2e-6}
NAMES = {1: "fp16x2", 2: "bf16x2", 3: "bf16x3"}


def stress_input(batch, n, seed):
    x = rand_c64((batch, n), seed)
    rng = np.random.default_rng(seed + 1)
    mask = rng.random((batch, n)) < 0.01
    x[mask] *= 1000
    return x


def choice(split, mode=0):
    return [mode, -1, -1, -1, -1, -1, -1, -1, 0, 0, 0, split]


@pytest.mark.parametrize("split", [1, 2, 3])
@pytest.mark.parametrize("logn", [4, 5, 6, 7, 9, 11, 12, 13])
def test_split_single_tile(emu, split, logn):
    n = 1 << logn
    x = stress_input(3, n, 100 + logn)
    for sign in (-1, +1):
        rc, msg, y = emu_run(emu, n, 3, x, sign, choice(split))
        assert rc == 0, msg
        e = oracle.rel_l2(y, oracle.fft(x, sign)).max()
        assert e < TOL[split], (NAMES[split], logn, sign, e)
    d = describe(emu, n, 3, choice(split))
    assert d["precision"] == NAMES[split] and d["kernels"][0]["tc"] == 1


@pytest.mark.parametrize("split", [1, 3])
@pytest.mark.parametrize("logn", [14, 15, 17])
def test_split_four_step(emu, split, logn):
    n = 1 << logn
    x = stress_input(2, n, 200 + logn)
    rc, msg, y = emu_run(emu, n, 2, x, -1, choice(split))
    assert rc == 0, msg
    assert oracle.rel_l2(y, oracle.fft(x, -1)).max() < TOL[split]
    d = describe(emu, n, 2, choice(split))
    assert [k["kind"] for k in d["kernels"]] == ["col", "row"] and all(k["tc"] == 1 for k in d["kernels"])


def test_split_small_sizes_run_fp32_tiles(emu):
    """n < 16 has no radix-16 pass: the split plan runs the FP32 tile."""
    for logn in range(0, 4):
        n = 1 << logn
        x = rand_c64((5, n), logn)
        rc, msg, y = emu_run(emu, n, 5, x, -1, choice(1))
        assert rc == 0, msg
        assert oracle.rel_l2(y, oracle.fft(x, -1)).max() < 1e-6


def test_split_rejects_persistent_variants(emu):
    """Split precision runs the plain single / four-step tiles: a request for
    the bulk-load variants is refused."""
    n = 1 << 16
    x = rand_c64((1, n), 1)
    rc, msg, _ = emu_run(emu, n, 1, x, -1, [2, -1, -1, -1, -1, -1, -1, -1, 0, 0, 2, 1])
    assert rc == 2 and "split precision" in msg


def test_host_16bit_conversions_match_numpy(emu):
    """The emulator's fp16 / bf16 rounding (round to nearest even, fp16
    subnormals) against numpy's float16 and a bit-level bf16 reference."""
    emu.emu_to16.restype = ctypes.c_uint
    emu.emu_to16.argtypes = [ctypes.c_float, ctypes.c_int]
    emu.emu_from16.restype = ctypes.c_float
    emu.emu_from16.argtypes = [ctypes.c_uint, ctypes.c_int]
    rng = np.random.default_rng(7)
    vals = np.concatenate([
        rng.standard_normal(2000).astype(np.float32) * np.float32(10.0) ** rng.integers(-9, 5, 2000),
        np.float32([0.0, -0.0, 1.0, -1.0, 65504.0, 6.1035156e-05, 5.9604645e-08, 2.9802322e-08, 1.0009766,
                    1.0004883, 1.0014648, 0.33333334, 3.0517578e-05 * 1.5]),
    ]).astype(np.float32)
    for v in vals:
        h = emu.emu_to16(float(v), 0)
        assert h == int(np.float16(v).view(np.uint16)), (v, h)
        assert emu.emu_from16(h, 0) == np.float32(np.float16(v))
        u = int(np.float32(v).view(np.uint32))
        want = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF
        assert emu.emu_to16(float(v), 1) == want
        assert emu.emu_from16(want, 1) == np.uint32(want << 16).view(np.float32)
