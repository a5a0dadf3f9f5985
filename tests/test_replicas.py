"""The N > 1 path of bench.py: one process per GPU running the same fixed
per-GPU workload (replicas: every transform is independent, nothing is
exchanged).  Two gloo ranks on the CPU check the whole-job aggregation
(max over ranks of the timed region, value = world * bytes * steps / time)
and that the reference arm runs on rank 0 only."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 100.0 + 50.0 * rank  # rank 1 is slower: the job takes its time
        value, ms = bench.replica_value(local_ms, world, bytes_per_step=2e9, steps=4, device="cpu")
        q.put((rank, value, ms))
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregation():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29000 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, ms in got:
        assert ms == pytest.approx(150.0)
        assert value == pytest.approx(2 * 2e9 * 4 / 0.150 / 1e9)


def test_single_rank_value():
    sys.path.insert(0, ROOT)
    import bench
    value, ms = bench.replica_value(200.0, 1, bytes_per_step=1e9, steps=2, device="cpu")
    assert ms == 200.0 and value == pytest.approx(10.0)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_cpu_library_baselines_are_labelled():
    """cpu_baseline.libraries: FFTW3 single precision is either timed or
    reported unavailable, scipy.fft and the FP64 oracle carry GB/s."""
    sys.path.insert(0, ROOT)
    import bench
    libs = bench.cpu_library_sample([10, 12], 2, budget_s=0.05)
    assert libs["unit"] == "GB/s"
    f = libs["fftw3f_estimate"]
    assert (isinstance(f, float) and f > 0) or f.startswith("unavailable")
    assert libs["oracle_fp64"] > 0
    s = libs["scipy_fft_c64"]
    assert (isinstance(s, float) and s > 0) or s.startswith("unavailable")
