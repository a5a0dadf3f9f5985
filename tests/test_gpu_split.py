"""GPU parity of the split-precision tensor-core path (ESTL_PREC_SPLIT_*):
every radix-16 stage as mma.sync m16n8k16 GEMMs on 16-bit split operands with
FP32 accumulation, through the C ABI, against the FP64 oracle on inputs with
1% of the entries scaled by 1e3.

Tolerances (relative L2 per transform): fp16 hi+lo and bf16 hi+mid+lo within
the FP32 target 2e-6; bf16 hi+lo (16 significant bits) within 3e-5.  The
tensor-core kernels must be the ones that ran: the plan description names
them and the launch count matches.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = {1: 2e-6, 2: 3e-5, 3: 2e-6}


def stress(batch, n, seed):
    rng = np.random.default_rng(seed)
    x = (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(np.complex64)
    x[rng.random((batch, n)) < 0.01] *= 1000
    return x


@pytest.mark.parametrize("split", [1, 2, 3])
@pytest.mark.parametrize("logn", [4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 16, 18, 20, 22, 24])
def test_split_parity(engine, split, logn):
    import torch
    n = 1 << logn
    batch = max(1, min(6, (1 << 22) // n))
    x = stress(batch, n, 500 + 7 * logn + split)
    xd = torch.from_numpy(x).cuda()
    for direction in (-1, +1):
        p = engine.Plan(n, batch, direction, precision=split)
        d = p.describe()
        assert d["precision"] == {1: "fp16x2", 2: "bf16x2", 3: "bf16x3"}[split]
        assert all(k["tc"] == 1 for k in d["kernels"])
        y = p.execute(xd)
        torch.cuda.synchronize()
        e = oracle.rel_l2(y.cpu().numpy(), oracle.fft(x, direction)).max()
        assert e < TOL[split], (split, logn, direction, e)


def test_split_same_alone_and_batched(engine):
    """A transform gives the same result alone and inside a batch (the
    tensor-core tiles mix butterflies of several transforms in one warp)."""
    import torch
    n = 1 << 10
    x = stress(16, n, 9)
    xd = torch.from_numpy(x).cuda()
    yb = engine.Plan(n, 16, -1, precision=1).execute(xd)
    y5 = engine.Plan(n, 1, -1, precision=1).execute(xd[5:6].contiguous())
    torch.cuda.synchronize()
    assert torch.equal(yb[5:6], y5)
