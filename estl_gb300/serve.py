"""Python client of the serving loop (estl_serve_* in include/estl_cuda.h)."""
import ctypes

from ._lib import REQ_CONV, REQ_FFT, ServeConfig, ServeRequest, ServeResult, ServeStats, check, lib


class Server:
    """Continuous-batching server for FFT and FFT-convolution requests.

    Host arrays passed to submit_* must stay alive until poll() returns for
    that ticket (the server keeps a reference until then)."""

    def __init__(self, hbm_budget_bytes=0, max_inflight_batches=4, max_batch_requests=256, max_queue=0):
        cfg = ServeConfig(int(hbm_budget_bytes), int(max_inflight_batches), int(max_batch_requests), int(max_queue))
        h = ctypes.c_void_p()
        check(lib().estl_serve_start(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._keep = {}

    def _submit(self, req, keep):
        t = ctypes.c_uint64()
        check(lib().estl_serve_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        self._keep[t.value] = keep
        return t.value

    def submit_conv(self, signal, filt, out, flags=0):
        """signal, filt, out: contiguous float32 numpy arrays; flags: CONV_* bits,
        plus conv_precision(PREC_SPLIT_*) for the tensor-core FFT stages; out
        holds estl_conv_output_length floats."""
        from . import _check_host
        _check_host(signal, "float32", 0, "signal")  # lengths themselves are checked by the server
        _check_host(filt, "float32", 0, "filter")
        need = int(lib().estl_conv_output_length(signal.size, filt.size, int(flags)))
        _check_host(out, "float32", need, "out", writable=True)
        r = ServeRequest(REQ_CONV, 0, int(flags), 0, 0, signal.size, filt.size, signal.ctypes.data, filt.ctypes.data,
                         out.ctypes.data)
        return self._submit(r, (signal, filt, out))

    def submit_fft(self, x, out, direction=-1, precision=0):
        """x, out: contiguous complex64 numpy arrays of one power-of-two length;
        precision: PREC_FP32 or a PREC_SPLIT_* tensor-core form."""
        from . import _check_host
        _check_host(x, "complex64", 0, "x")
        _check_host(out, "complex64", x.size, "out", writable=True)
        r = ServeRequest(REQ_FFT, int(direction), int(precision) << 8, 0, x.size, 0, 0, x.ctypes.data, None,
                         out.ctypes.data)
        return self._submit(r, (x, out))

    def poll(self, ticket, timeout_ms=60000):
        """Waits for a request; returns its ServeResult (latency in microseconds)."""
        res = ServeResult()
        st = lib().estl_serve_poll(self._h, ctypes.c_uint64(ticket), int(timeout_ms), ctypes.byref(res))
        if st == 6:  # ESTL_TIMEOUT: the ticket stays valid
            return None
        self._keep.pop(ticket, None)
        check(st)
        return res

    def stats(self):
        s = ServeStats()
        check(lib().estl_serve_stats_get(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in ServeStats._fields_}

    def stop(self):
        if self._h:
            check(lib().estl_serve_stop(self._h))
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass
