"""estl_gb300 — GB300-native (sm_103a) FFT engine with ESTL's plugin semantics.

The engine is the C-ABI library libestl_cuda.so (include/estl_cuda.h); this
package is its Python binding.  PyTorch provides device memory and streams:

    import torch, estl_gb300 as estl
    estl.init()
    x = torch.randn(256, 4096, dtype=torch.complex64, device="cuda")
    y = estl.fft(x)                      # forward, unnormalised (FFTW_FORWARD)
    z = estl.fft(y, inverse=True) / 4096  # round trip

Plan objects mirror the reference's FFT<D> objects (FFT.h:19-36): a plan is
created for (size, batchCount, forward) and executed repeatedly.
"""
import ctypes
import json

from ._lib import (BACKWARD, FORWARD, LAYOUT_BLOCK_PLANAR, LAYOUT_INTERLEAVED, LAYOUT_SPLIT, PREC_FP32,
                   PREC_SPLIT_BF16, PREC_SPLIT_BF16X3, PREC_SPLIT_FP16, EstlError,
                   PlanOptions, check, lib)

__all__ = ["init", "shutdown", "Plan", "Plan2D", "Conv2DPlan", "PackedPlan", "fft", "fft_packed", "autotune",
           "max_batch", "memory_usage", "EstlError", "FORWARD", "BACKWARD", "CONV_CORRELATE",
           "CONV_REFERENCE_COMPAT"]

_initialised = False


def init(device=0, hbm_budget_bytes=0):
    """Select the CUDA device and set the engine's HBM budget (0 = 90% of free)."""
    global _initialised
    check(lib().estl_init(int(device), int(hbm_budget_bytes)))
    _initialised = True


def shutdown():
    global _initialised
    _plan_cache.clear()
    check(lib().estl_shutdown())
    _initialised = False


def _ensure_init():
    if not _initialised:
        init()


def max_batch(n):
    """FFT_OpenCL_Contiguous::getMaxBatchSize equivalent against the HBM budget."""
    _ensure_init()
    return int(lib().estl_max_batch(int(n)))


def memory_usage():
    used, budget = ctypes.c_size_t(), ctypes.c_size_t()
    check(lib().estl_memory_usage(ctypes.byref(used), ctypes.byref(budget)))
    return used.value, budget.value


def _check_host(a, dtype, numel, what, writable=False):
    """A host buffer handed to the library by pointer: a C-contiguous numpy
    array of `dtype` with at least `numel` elements."""
    import numpy as np
    if (not isinstance(a, np.ndarray) or a.dtype != np.dtype(dtype) or not a.flags.c_contiguous or a.size < numel
            or (writable and not a.flags.writeable)):
        raise EstlError(1, f"{what} must be a C-contiguous{' writable' if writable else ''} "
                           f"{np.dtype(dtype).name} numpy array of >= {numel} elements")


def _stream_handle(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Plan:
    """`batch` transforms of length n, forward (-1) or backward (+1)."""

    MODES = {"auto": 0, "single": 1, "four_step": 2, "three_pass": 4}

    TILE_FIELDS = ("split_log2", "single_loge", "single_logc", "col_loge", "col_logc", "row_loge", "row_logc",
                   "pipelined", "split2_log2", "single_logr", "col_logr", "row_logr", "single_cluster_log2")

    def __init__(self, n, batch=1, direction=FORWARD, precision=PREC_FP32, mode="auto", chunk=0, tiles=None):
        """tiles: optional dict of estl_plan_options tile fields (split_log2, col_loge, ...; modes
        single / four_step / three_pass), missing ones left to the planner."""
        _ensure_init()
        self.n, self.batch, self.direction = int(n), int(batch), int(direction)
        h = ctypes.c_void_p()
        opts = PlanOptions(self.MODES[mode] if isinstance(mode, str) else int(mode), 0, int(chunk))
        if tiles:
            unknown = set(tiles) - set(self.TILE_FIELDS)
            if unknown:
                raise EstlError(1, f"unknown tile fields {sorted(unknown)}")
            opts.explicit_tiles = 1
            for f in self.TILE_FIELDS:
                setattr(opts, f, int(tiles.get(f, -1)))
        check(lib().estl_plan_create_ex(self.n, self.batch, self.direction, int(precision), ctypes.byref(opts),
                                        ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def describe(self):
        buf = ctypes.create_string_buffer(2048)
        check(lib().estl_plan_describe(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def check(self):
        """Synchronise; raise if a persistent kernel's bounded copy wait gave up."""
        check(lib().estl_plan_check(self._h))

    @property
    def launches(self):
        return int(lib().estl_plan_launches(self._h))

    def execute_ptr(self, d_in, d_out, stream=0):
        """Device pointers (ints) of n*batch complex64 elements."""
        check(lib().estl_execute(self._h, ctypes.c_void_p(d_in), ctypes.c_void_p(d_out), ctypes.c_void_p(stream)))

    def execute(self, x, out=None, stream=None):
        """x: contiguous complex64 CUDA tensor with n*batch elements."""
        import torch
        if x.dtype != torch.complex64 or not x.is_cuda or not x.is_contiguous():
            raise EstlError(1, "input must be a contiguous complex64 CUDA tensor")
        if x.numel() != self.n * self.batch:
            raise EstlError(1, f"input has {x.numel()} elements, plan expects {self.n * self.batch}")
        if out is None:
            out = torch.empty_like(x)
        if out.dtype != torch.complex64 or not out.is_cuda or not out.is_contiguous() or out.numel() != x.numel():
            raise EstlError(1, f"output must be a contiguous complex64 CUDA tensor of {x.numel()} elements")
        self.execute_ptr(x.data_ptr(), out.data_ptr(), _stream_handle(stream))
        return out

    def execute_layout(self, x, layout, out=None, stream=None):
        """x: float32 CUDA tensor holding the batch in `layout` (LAYOUT_BLOCK_PLANAR /
        LAYOUT_SPLIT / LAYOUT_INTERLEAVED), layout_floats(layout, n * batch) floats."""
        import torch
        floats = int(lib().estl_layout_floats(int(layout), self.n * self.batch))
        if floats < 0:
            raise EstlError(1, f"unknown layout {layout}")
        if x.dtype != torch.float32 or not x.is_cuda or not x.is_contiguous() or x.numel() < floats:
            raise EstlError(1, f"input must be a contiguous float32 CUDA tensor of >= {floats} floats")
        if out is None:
            out = torch.zeros(floats, dtype=torch.float32, device=x.device)
        if out.dtype != torch.float32 or not out.is_cuda or not out.is_contiguous() or out.numel() < floats:
            raise EstlError(1, f"output must be a contiguous float32 CUDA tensor of >= {floats} floats")
        check(lib().estl_execute_layout(self._h, int(layout), ctypes.c_void_p(x.data_ptr()),
                                        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(_stream_handle(stream))))
        return out

    def execute_host_layout(self, x, out, layout):
        """Host float32 numpy arrays in `layout` (see execute_layout)."""
        floats = int(lib().estl_layout_floats(int(layout), self.n * self.batch))
        if floats < 0:
            raise EstlError(1, f"unknown layout {layout}")
        _check_host(x, "float32", floats, "input")
        _check_host(out, "float32", floats, "output", writable=True)
        check(lib().estl_execute_host_layout(self._h, int(layout), ctypes.c_void_p(x.ctypes.data),
                                             ctypes.c_void_p(out.ctypes.data)))
        return out

    def execute_host(self, x, out):
        """Host numpy complex64 arrays (pinned memory recommended)."""
        _check_host(x, "complex64", self.n * self.batch, "input")
        _check_host(out, "complex64", self.n * self.batch, "output", writable=True)
        check(lib().estl_execute_host(self._h, ctypes.c_void_p(x.ctypes.data), ctypes.c_void_p(out.ctypes.data)))
        return out

    KERNEL_KINDS = ("single", "col", "row", "copy", "unused", "column")

    def set_profiling(self, enable=True):
        """Bracket every launch with CUDA events (per-kernel timers)."""
        check(lib().estl_plan_set_profiling(self._h, 1 if enable else 0))

    def kernel_stats(self):
        """{kind: (launches, total_ms, algorithmic_bytes)} of profiled launches."""
        k = len(self.KERNEL_KINDS)
        L = (ctypes.c_int64 * k)()
        T = (ctypes.c_double * k)()
        B = (ctypes.c_double * k)()
        check(lib().estl_plan_kernel_stats(self._h, L, T, B))
        return {k: (int(L[i]), float(T[i]), float(B[i])) for i, k in enumerate(self.KERNEL_KINDS) if L[i]}

    def close(self):
        if getattr(self, "_h", None):
            lib().estl_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan2D(Plan):
    """`batch` 2D transforms of ydim rows by xdim columns (row-major, x fastest):
    the layout of ESTL's FFT2D<D>.  Powers of two, ydim <= 2^12, FP32."""

    def __init__(self, xdim, ydim, batch=1, direction=FORWARD):
        _ensure_init()
        self.xdim, self.ydim = int(xdim), int(ydim)
        self.n, self.batch, self.direction = self.xdim * self.ydim, int(batch), int(direction)
        h = ctypes.c_void_p()
        check(lib().estl_plan2d_create(self.xdim, self.ydim, self.batch, self.direction, PREC_FP32, ctypes.byref(h)))
        self._h = h


CONV_CORRELATE = 1
CONV_REFERENCE_COMPAT = 2


class Conv2DPlan:
    """2D FFT convolution of `count` real images (height x width, row-major)
    with one real filter (kheight x kwidth), after Convolution2D_FFT::convolve
    (Convolution.h:95-148).  flags: CONV_CORRELATE, CONV_REFERENCE_COMPAT (the
    reference's centred, K^[0]-normalised height x width result; default: the
    full linear convolution)."""

    def __init__(self, width, height, kwidth, kheight, count=1, flags=0):
        _ensure_init()
        self.width, self.height, self.kwidth, self.kheight = int(width), int(height), int(kwidth), int(kheight)
        self.count, self.flags = int(count), int(flags)
        ow, oh = ctypes.c_int64(), ctypes.c_int64()
        check(lib().estl_conv2d_output_size(self.width, self.height, self.kwidth, self.kheight, self.flags,
                                            ctypes.byref(ow), ctypes.byref(oh)))
        self.out_width, self.out_height = ow.value, oh.value
        h = ctypes.c_void_p()
        check(lib().estl_conv2d_plan_create(self.width, self.height, self.kwidth, self.kheight, self.count,
                                            self.flags, ctypes.byref(h)))
        self._h = h

    @staticmethod
    def _check_tensor(x, numel, what):
        import torch
        if x.dtype != torch.float32 or not x.is_cuda or not x.is_contiguous() or x.numel() != numel:
            raise EstlError(1, f"{what} must be a contiguous float32 CUDA tensor of {numel} elements")

    def set_filter(self, k, stream=None):
        """k: float32 CUDA tensor of kheight * kwidth elements."""
        self._check_tensor(k, self.kwidth * self.kheight, "filter")
        check(lib().estl_conv2d_plan_set_filter(self._h, ctypes.c_void_p(k.data_ptr()), _stream_handle(stream)))

    def execute(self, images, out=None, stream=None):
        """images: float32 CUDA tensor of count * height * width elements; returns
        (count, out_height, out_width)."""
        import torch
        self._check_tensor(images, self.count * self.width * self.height, "images")
        if out is None:
            out = torch.empty((self.count, self.out_height, self.out_width), dtype=torch.float32,
                              device=images.device)
        self._check_tensor(out, self.count * self.out_width * self.out_height, "out")
        check(lib().estl_conv2d_plan_execute(self._h, ctypes.c_void_p(images.data_ptr()),
                                             ctypes.c_void_p(out.data_ptr()), _stream_handle(stream)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().estl_conv2d_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PackedPlan:
    """An uneven batch: transform i of length sizes[i] (a power of two in
    [2, 2^18]) at complex-element offset offsets[i] of both the input and the
    output buffer, transforms not overlapping.  mode "persistent": one launch
    whose CTAs take work items from a device queue; "per_size": one launch per
    size class; "bucketed": the engine's own plan per length.  The reference
    has one FFT object per size (tests/Test.cpp:45-60).

    convolutions: optional (n, 5) integers per FFT convolution -- signal
    length, filter length, and the signal, filter and output offsets in
    floats (estl_conv_request) -- run in the same plan (a mixed batch,
    estl_packed_mixed_plan_create) with conv_flags (CONV_CORRELATE,
    CONV_REFERENCE_COMPAT, ...); offsets / sizes may then be empty.  A mixed
    plan runs through execute_mixed."""

    MODES = {"persistent": 0, "per_size": 1, "bucketed": 2}

    def __init__(self, offsets, sizes, direction=FORWARD, mode="persistent", convolutions=None, conv_flags=0):
        import numpy as np
        self._offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        self._sizes = np.ascontiguousarray(sizes, dtype=np.int64)
        mixed = convolutions is not None
        if self._offsets.ndim != 1 or self._offsets.shape != self._sizes.shape or (
                self._sizes.size == 0 and not mixed):
            raise EstlError(1, "offsets and sizes must be 1-D arrays of one non-zero length")
        if mode not in self.MODES:
            raise EstlError(1, f"mode must be one of {sorted(self.MODES)}")
        if mixed:
            self._convs = np.ascontiguousarray(convolutions, dtype=np.int64).reshape(-1, 5)
        _ensure_init()
        self.direction = int(direction)
        self.extent = int((self._offsets + self._sizes).max()) if self._sizes.size else 0
        h = ctypes.c_void_p()
        if mixed:
            check(lib().estl_packed_mixed_plan_create(self._offsets.ctypes.data, self._sizes.ctypes.data,
                                                      self._sizes.size, self.direction, self._convs.ctypes.data,
                                                      len(self._convs), int(conv_flags), self.MODES[mode],
                                                      ctypes.byref(h)))
        else:
            check(lib().estl_packed_plan_create(self._offsets.ctypes.data, self._sizes.ctypes.data, self._sizes.size,
                                                self.direction, self.MODES[mode], ctypes.byref(h)))
        self._h = h
        # floats the signal, filter and output arrays must hold (0 without convolutions)
        d = self.describe()
        self.conv_extents = (d.get("conv_signal_floats", 0), d.get("conv_filter_floats", 0),
                             d.get("conv_out_floats", 0))

    def execute_mixed(self, x, out, signals, filters, conv_out, stream=None):
        """A mixed batch: x / out as execute (None when there are no
        transforms); signals, filters, conv_out: contiguous float32 CUDA
        tensors holding the convolutions' offsets, of at least
        conv_extents floats each."""
        import torch
        for name, t, need in zip(("signals", "filters", "conv_out"), (signals, filters, conv_out), self.conv_extents):
            if need and t is None:
                raise EstlError(1, f"{name} is required: the plan has convolutions")
            if t is not None and (t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous()
                                  or t.numel() < need):
                raise EstlError(1, f"{name} must be a contiguous float32 CUDA tensor of >= {need} elements")
        for name, t in (("x", x), ("out", out)):
            if t is not None and (t.dtype != torch.complex64 or not t.is_cuda or not t.is_contiguous()
                                  or t.numel() < self.extent):
                raise EstlError(1, f"{name} must be a contiguous complex64 CUDA tensor of >= {self.extent} elements")
        ptr = lambda t: ctypes.c_void_p(t.data_ptr() if t is not None else None)  # noqa: E731
        check(lib().estl_packed_mixed_execute(self._h, ptr(x), ptr(out), ptr(signals), ptr(filters), ptr(conv_out),
                                              ctypes.c_void_p(_stream_handle(stream))))
        return out, conv_out

    def execute(self, x, out=None, stream=None):
        """x: contiguous complex64 CUDA tensor of at least `extent` elements;
        out (same size as x) receives the transforms, the gaps between them
        are not written."""
        import torch
        if x.dtype != torch.complex64 or not x.is_cuda or not x.is_contiguous() or x.numel() < self.extent:
            raise EstlError(1, f"input must be a contiguous complex64 CUDA tensor of >= {self.extent} elements")
        if out is None:
            out = torch.empty_like(x)
        if out.dtype != torch.complex64 or not out.is_cuda or not out.is_contiguous() or out.numel() < self.extent:
            raise EstlError(1, f"output must be a contiguous complex64 CUDA tensor of >= {self.extent} elements")
        check(lib().estl_packed_execute(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                        ctypes.c_void_p(_stream_handle(stream))))
        return out

    def check(self):
        """Synchronise; raise if a row item's dependency wait gave up."""
        check(lib().estl_packed_check(self._h))

    def describe(self):
        buf = ctypes.create_string_buffer(8192)
        check(lib().estl_packed_plan_describe(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def close(self):
        if getattr(self, "_h", None):
            lib().estl_packed_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fft_packed(x, offsets, sizes, inverse=False, out=None, stream=None):
    """One blocking call for an uneven batch used once (estl_execute_packed):
    plan, execute, wait, check and release.  Arguments as PackedPlan."""
    import numpy as np
    import torch
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    sizes = np.ascontiguousarray(sizes, dtype=np.int64)
    if offsets.ndim != 1 or offsets.shape != sizes.shape or sizes.size == 0:
        raise EstlError(1, "offsets and sizes must be 1-D arrays of one non-zero length")
    extent = int((offsets + sizes).max())
    if x.dtype != torch.complex64 or not x.is_cuda or not x.is_contiguous() or x.numel() < extent:
        raise EstlError(1, f"input must be a contiguous complex64 CUDA tensor of >= {extent} elements")
    _ensure_init()
    if out is None:
        out = torch.empty_like(x)
    if out.dtype != torch.complex64 or not out.is_cuda or not out.is_contiguous() or out.numel() < extent:
        raise EstlError(1, f"output must be a contiguous complex64 CUDA tensor of >= {extent} elements")
    check(lib().estl_execute_packed(offsets.ctypes.data, sizes.ctypes.data, sizes.size,
                                    BACKWARD if inverse else FORWARD, ctypes.c_void_p(x.data_ptr()),
                                    ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(_stream_handle(stream))))
    return out


_plan_cache = {}


def fft(x, inverse=False, out=None, stream=None):
    """Batched FFT over the last dimension of a complex64 CUDA tensor."""
    n = x.shape[-1]
    batch = x.numel() // n
    key = (n, batch, BACKWARD if inverse else FORWARD)
    p = _plan_cache.get(key)
    if p is None:
        p = _plan_cache[key] = Plan(n, batch, key[2])
    return p.execute(x.contiguous(), out=out, stream=stream)


def autotune(n, batch, iters=5):
    """Time every candidate plan for (n, batch); cache and return the best."""
    _ensure_init()
    buf = ctypes.create_string_buffer(1 << 16)
    check(lib().estl_autotune(int(n), int(batch), int(iters), buf, len(buf)))
    for key in [k for k in _plan_cache if k[0] == n and k[1] == batch]:
        _plan_cache.pop(key).close()
    return json.loads(buf.value.decode())
