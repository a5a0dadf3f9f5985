"""Small, self-contained FFT launches for profiling one kernel at a time.

    python -m estl_gb300.profile_cases <case> [<case> ...]

Each case plans one transform size on a batch of 2^24 complex64 elements
(128 MiB per buffer: larger than the L2, small enough for a profiler's
replays), executes it three times and checks the plan's device status, so
that a profiler capture of launch 2 (`-s 1 -c 1`) sees a warm kernel.
Cases: the planner default for a size (`n13`, `n14`, ... `n24`), an
explicit tile from CASES below, a length that is not a power of two
(`len1000`: Bluestein), or `mixed` (a packed batch of transforms and FFT
convolutions, estl_packed_mixed_*).
"""
import sys

CASES = {
    # one transform per thread-block cluster (cluster_core.cuh)
    "cluster15": (15, dict(mode="single", tiles={"single_loge": 4, "single_cluster_log2": 3, "split_log2": 8})),
    "cluster16": (16, dict(mode="single", tiles={"single_loge": 4, "single_cluster_log2": 3, "split_log2": 8})),
    # whole transforms in one CTA (fft_core.cuh SingleKernel, radix 32)
    "single13": (13, dict(mode="single", tiles={"single_loge": 5, "single_logc": 0, "single_logr": 5})),
    "single14": (14, dict(mode="single", tiles={"single_loge": 5, "single_logc": 0, "single_logr": 5})),
    # the plain 4096 x 256 configuration (one small batch, latency-bound)
    "c1": (12, dict(batch=256)),
}


def run_mixed():
    """4096 transforms of 2^6..2^12 and 4096 real FFT convolutions of padded
    length 2^6..2^12 (the packed kernel's work items), persistent mode."""
    import numpy as np
    import torch

    import estl_gb300 as estl
    rng = np.random.default_rng(1)
    sizes = (1 << rng.integers(6, 13, 4096)).astype(np.int64)
    offsets = np.concatenate([[0], np.cumsum(sizes[:-1])]).astype(np.int64)
    reqs, so, fo, oo = [], 0, 0, 0
    for lg in rng.integers(6, 13, 4096):
        total = int(rng.integers((1 << (lg - 1)) + 1, (1 << lg) + 1))
        k = int(rng.integers(1, total // 4 + 2))
        reqs.append((total - k + 1, k, so, fo, oo))
        so, fo, oo = so + total - k + 1, fo + k, oo + total
    x = torch.randn(int(sizes.sum()), dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    sig, filt = torch.randn(so, device="cuda"), torch.randn(fo, device="cuda")
    out = torch.empty(oo, device="cuda")
    p = estl.PackedPlan(offsets, sizes, estl.FORWARD, "persistent", convolutions=reqs)
    for _ in range(3):
        p.execute_mixed(x, y, sig, filt, out)
    p.check()
    print("mixed", p.describe(), flush=True)
    p.close()


def run(case, elements_log=24):
    import torch

    import estl_gb300 as estl
    if case == "mixed":
        return run_mixed()
    if case.startswith("len") and case[3:].isdigit():
        estl.init(0)
        n = int(case[3:])
        batch = max(1, (1 << elements_log) // n)
        x = torch.view_as_complex((torch.rand((n * batch, 2), device="cuda") * 2 - 1).contiguous())
        p = estl.Plan(n, batch, estl.FORWARD)
        y = torch.empty_like(x)
        for _ in range(3):
            p.execute(x, out=y)
        torch.cuda.synchronize()
        p.check()
        print(case, p.describe(), flush=True)
        return p.close()
    if case in CASES:
        logn, kw = CASES[case]
        kw = dict(kw)
    elif case.startswith("n") and case[1:].isdigit():
        logn, kw = int(case[1:]), {}
    else:
        raise SystemExit(f"unknown case {case!r}; known: {sorted(CASES)} or n<log2 N>")
    estl.init(0)
    n = 1 << logn
    batch = kw.pop("batch", max(1, (1 << elements_log) // n))
    x = torch.view_as_complex((torch.rand((n * batch, 2), device="cuda") * 2 - 1).contiguous())
    y = torch.empty_like(x)
    p = estl.Plan(n, batch, estl.FORWARD, **kw)
    for _ in range(3):
        p.execute(x, out=y)
    torch.cuda.synchronize()
    p.check()
    print(case, p.describe(), flush=True)
    p.close()


if __name__ == "__main__":
    for c in sys.argv[1:]:
        run(c)
