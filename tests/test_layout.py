"""Other host layouts of the complex data (f3): block-planar
(PlannarizedComplexArray<5, D>, the layout of FFT_OpenCL_Contiguous:
blocks of 32 real parts then 32 imaginary parts, Complex.h:34-48,97-130) and
split (all real parts, then all imaginary parts: ComplexArray(n, true)).

The conversions are exact moves, so a transform through
estl_execute_layout / estl_execute_host_layout must be bit-identical to the
interleaved execution of the same plan.  The index rule is restated here
(to_layout / from_layout) from the reference's ArrayPlannarizer::getPosition
(Complex.h:41-43): position = ((i >> 5) << 6) | (element << 5) | (i & 31).
"""
import numpy as np
import pytest

BLOCK_PLANAR, SPLIT = 1, 2


def layout_floats(layout, total):
    if layout == SPLIT:
        return 2 * total
    return (((total - 1) >> 5) << 6) + 32 + ((total - 1) & 31) + 1


def positions(layout, total):
    i = np.arange(total, dtype=np.int64)
    if layout == SPLIT:
        return i, i + total
    re = ((i >> 5) << 6) | (i & 31)
    return re, re + 32


def to_layout(x, layout):
    flat = x.reshape(-1)
    out = np.full(layout_floats(layout, flat.size), np.nan, np.float32)
    re, im = positions(layout, flat.size)
    out[re] = flat.real
    out[im] = flat.imag
    return out


def from_layout(a, layout, shape):
    total = int(np.prod(shape))
    re, im = positions(layout, total)
    return (a[re] + 1j * a[im]).astype(np.complex64).reshape(shape)


def test_layout_index_rule_is_a_bijection():
    for total in (1, 31, 32, 40, 1000):
        re, im = positions(BLOCK_PLANAR, total)
        allpos = np.concatenate([re, im])
        assert len(np.unique(allpos)) == 2 * total
        assert allpos.max() + 1 == layout_floats(BLOCK_PLANAR, total)


def rand_c64(shape, seed):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64)


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [BLOCK_PLANAR, SPLIT])
@pytest.mark.parametrize("n,batch", [(8, 5), (1, 7), (4096, 33), (1 << 16, 3), (1 << 20, 2), (64, 1)])
def test_gpu_layout_device_and_host(engine, layout, n, batch):
    import torch
    x = rand_c64((batch, n), n + batch + layout)
    for direction in (-1, +1):
        p = engine.Plan(n, batch, direction)
        ref = p.execute(torch.from_numpy(x).cuda()).cpu().numpy()
        a = to_layout(x, layout)
        assert int(engine.lib().estl_layout_floats(layout, n * batch)) == a.size
        y = p.execute_layout(torch.from_numpy(a).cuda(), layout).cpu().numpy()
        assert np.array_equal(from_layout(y, layout, x.shape), ref)
        h = np.full(a.size, np.nan, np.float32)
        p.execute_host_layout(a, h, layout)
        assert np.array_equal(from_layout(h, layout, x.shape), ref)
        assert not np.isnan(h).any()


@pytest.mark.gpu
def test_gpu_layout_2d(engine):
    import torch
    x = rand_c64((3, 64, 128), 9)
    p = engine.Plan2D(128, 64, 3, -1)
    ref = p.execute(torch.from_numpy(x).cuda()).cpu().numpy()
    for layout in (BLOCK_PLANAR, SPLIT):
        a = to_layout(x, layout)
        y = p.execute_layout(torch.from_numpy(a).cuda(), layout).cpu().numpy()
        assert np.array_equal(from_layout(y, layout, x.shape), ref)


@pytest.mark.gpu
def test_gpu_layout_rejects_unknown(engine):
    import torch
    from estl_gb300 import EstlError
    p = engine.Plan(64, 2, -1)
    with pytest.raises(EstlError):
        p.execute_layout(torch.zeros(256, device="cuda"), 7)
