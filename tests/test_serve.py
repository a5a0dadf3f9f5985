"""The serving loop (estl_serve_*): FFT and FFT-convolution requests of mixed
lengths, continuous batching, HBM admission, and the same result alone and
in the mix."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.sum((a - b) ** 2) / max(np.sum(b ** 2), 1e-300)))


def conv_requests(count, seed):
    """Served-convolution configuration shapes: signal log-uniform 2^8..2^20,
    filter log-uniform 2^4..2^12, both N(0,1)."""
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(count):
        L = int(2 ** rng.uniform(8, 20))
        K = int(2 ** rng.uniform(4, 12))
        s = rng.standard_normal(L).astype(np.float32)
        f = rng.standard_normal(K).astype(np.float32)
        reqs.append((s, f))
    return reqs


NO_PAIRING = 4


def run_mixed(server, convs, ffts, precision=0, flags=0):
    tickets = []
    outs = []
    for s, f in convs:
        out = np.full(s.size + f.size - 1, np.nan, np.float32)
        tickets.append(server.submit_conv(s, f, out, flags=(precision << 8) | flags))
        outs.append(out)
    for x, d in ffts:
        out = np.full_like(x, np.nan)
        tickets.append(server.submit_fft(x, out, d, precision=precision))
        outs.append(out)
    results = [server.poll(t) for t in tickets]
    return outs, results


def test_mixed_requests_against_oracle(engine):
    from estl_gb300.serve import Server
    convs = conv_requests(40, 1)
    rng = np.random.default_rng(2)
    ffts = []
    for logn in (6, 10, 12, 15, 18, 20):
        x = (rng.standard_normal(1 << logn) + 1j * rng.standard_normal(1 << logn)).astype(np.complex64)
        ffts.append((x, -1 if logn % 2 else +1))
    srv = Server(max_inflight_batches=4, max_batch_requests=16)
    try:
        outs, results = run_mixed(srv, convs, ffts)
        stats = srv.stats()
    finally:
        srv.stop()
    for (s, f), out in zip(convs, outs[:len(convs)]):
        assert rel(out, oracle.conv_fft(s.astype(np.float64), f.astype(np.float64))) < 1e-6
    for (x, d), out in zip(ffts, outs[len(convs):]):
        assert oracle.rel_l2(out[None], oracle.fft(x[None], d))[0] < 2e-6
    assert all(r.status == 0 and r.latency_us > 0 for r in results)
    assert stats["completed"] == len(results) and stats["batches"] >= 3
    assert max(r.batch_requests for r in results) > 1


def test_split_precision_requests(engine):
    """The batched split-precision form (fp16 hi+lo tensor-core FFT stages) of
    the served convolution and FFT requests: same accuracy targets as FP32
    (1e-6 for convolutions, 2e-6 for transforms), and the same result alone
    and in the mix."""
    from estl_gb300 import PREC_SPLIT_FP16
    from estl_gb300.serve import Server
    convs = conv_requests(30, 4)
    rng = np.random.default_rng(5)
    ffts = [((rng.standard_normal(1 << l) + 1j * rng.standard_normal(1 << l)).astype(np.complex64), -1)
            for l in (8, 13, 16, 20)]
    srv = Server(max_inflight_batches=4, max_batch_requests=16)
    try:
        outs, results = run_mixed(srv, convs, ffts, precision=PREC_SPLIT_FP16)
    finally:
        srv.stop()
    for (s, f), out in zip(convs, outs[:len(convs)]):
        assert rel(out, oracle.conv_fft(s.astype(np.float64), f.astype(np.float64))) < 1e-6
    for (x, d), out in zip(ffts, outs[len(convs):]):
        assert oracle.rel_l2(out[None], oracle.fft(x[None], d))[0] < 2e-6
    assert all(r.status == 0 for r in results)
    srv = Server(max_inflight_batches=1, max_batch_requests=1)
    try:
        alone, _ = run_mixed(srv, [convs[11]], [], precision=PREC_SPLIT_FP16)
    finally:
        srv.stop()
    assert np.array_equal(alone[0], outs[11])


@pytest.mark.parametrize("pairing", [True, False])
def test_same_result_alone_and_in_the_mix(engine, pairing):
    """Every request of a mixed batch against the same request served alone
    (one request per batch, one batch in flight), and both against the FP64
    oracle at the stated 1e-6 tolerance.  Requests that run on their own
    (padded n > 2^14, or pairing switched off) are bit-identical alone and in
    the mix; a request of padded n <= 2^14 shares its complex transform with
    another request of the mix, so it differs from its lone result only by
    rounding, within the tolerance."""
    from estl_gb300.serve import Server
    flags = 0 if pairing else NO_PAIRING
    convs = conv_requests(24, 3)
    srv = Server(max_inflight_batches=3, max_batch_requests=32)
    try:
        mixed, results = run_mixed(srv, convs, [], flags=flags)
    finally:
        srv.stop()
    assert max(r.batch_requests for r in results) > 1
    srv = Server(max_inflight_batches=1, max_batch_requests=1)
    try:
        alone, alone_results = run_mixed(srv, convs, [], flags=flags)
    finally:
        srv.stop()
    assert all(r.batch_requests == 1 for r in alone_results)
    for i, (s, f) in enumerate(convs):
        ref = oracle.conv_fft(s.astype(np.float64), f.astype(np.float64))
        assert rel(mixed[i], ref) < 1e-6 and rel(alone[i], ref) < 1e-6, i
        assert rel(mixed[i], alone[i]) < 1e-6, i
        padded = 1 << int(np.ceil(np.log2(s.size + f.size - 1)))
        if not pairing or padded > 1 << 14:
            assert np.array_equal(alone[i], mixed[i]), (i, padded)


def test_admission_budget(engine):
    from estl_gb300 import EstlError
    from estl_gb300.serve import Server
    convs = conv_requests(30, 4)
    budget = 160 << 20
    srv = Server(hbm_budget_bytes=budget, max_inflight_batches=4, max_batch_requests=64)
    try:
        outs, results = run_mixed(srv, convs, [])
        st = srv.stats()
        assert st["max_inflight_bytes"] <= budget
        # a request that can never fit the budget is refused at submit time
        big = np.zeros((1 << 21) - 4096, np.float32)
        f = np.zeros(4096, np.float32)
        out = np.zeros(big.size + f.size - 1, np.float32)
        tiny = Server(hbm_budget_bytes=1 << 20)
        try:
            with pytest.raises(EstlError) as e:
                tiny.submit_conv(big, f, out)
            assert e.value.name == "ESTL_ADMISSION_REJECTED"
        finally:
            tiny.stop()
    finally:
        srv.stop()
    for (s, f), out in zip(convs, outs):
        assert rel(out, oracle.conv_fft(s.astype(np.float64), f.astype(np.float64))) < 1e-6


def test_submit_checks_host_arrays(engine):
    """The server copies results into the caller's host arrays by pointer, so
    submit refuses a short output, a wrong dtype or a read-only output before
    the request is queued; a well-formed request then runs as usual."""
    from estl_gb300 import EstlError
    from estl_gb300.serve import Server
    srv = Server(max_inflight_batches=1)
    try:
        s = np.ones(100, np.float32)
        f = np.ones(10, np.float32)
        ro = np.zeros(109, np.float32)
        ro.flags.writeable = False
        for bad in ((s, f, np.zeros(108, np.float32)), (s.astype(np.float64), f, np.zeros(109, np.float32)),
                    (s, f, ro)):
            with pytest.raises(EstlError):
                srv.submit_conv(*bad)
        with pytest.raises(EstlError):
            srv.submit_fft(np.zeros(64, np.complex64), np.zeros(63, np.complex64))
        out = np.full(109, np.nan, np.float32)
        res = srv.poll(srv.submit_conv(s, f, out))
        assert res.status == 0
        assert rel(out, oracle.conv_fft(s.astype(np.float64), f.astype(np.float64))) < 1e-6
        assert srv.stats()["submitted"] == 1  # the refused ones never reached the queue
    finally:
        srv.stop()
