"""GB300-native dilation-based Hausdorff distance for 3D binary masks.

Python mirror of the C ABI in include/hd/hd.h (libhd_gb300.so, hand-written
sm_103a kernels).  The reference's entry point is the C++ call
``HausdorffDistance::computeDistance(Volume*, Volume*)``
(forBench/HausdorffDistance.cuh:17); :class:`HausdorffDistance` and
:class:`Volume` below mirror it, and :class:`Context` exposes the rest
(device-resident inputs, batches, profiling, distance maps, autotuning) and
:class:`Server` the continuous-batching request loop.

Masks are ``(D, H, W)`` arrays (x fastest, like ``Volume``), numpy arrays or
torch tensors on the CPU or on the GPU; nonzero is foreground.  Metric names:
``"se6"`` (6-neighbour element, Manhattan distance) and ``"se18"`` (the
reference's default 18-neighbour element, forBench/HausdorffDistance.cu:35-58).
"""
from __future__ import annotations

import ctypes
from typing import Iterable, Sequence

import numpy as np

from . import _native as N
from ._native import (HD_EMPTY_MASK, HD_ERR_BAD_ARG, HD_ERR_BUSY, HD_ERR_CANCELLED, HD_ERR_CUDA,
                      HD_ERR_ITER_LIMIT, HD_ERR_NOT_READY, HD_ERR_OOM, HD_ERR_TIMEOUT,
                      HD_ERR_UNSUPPORTED, HD_OK, HD_SE6, HD_SE18_FORBENCH)

__all__ = [
    "Context", "PreparedBatch", "Server", "HausdorffDistance", "Volume", "HDError", "metric_code", "load_hdf5_bool",
    "HD_OK", "HD_EMPTY_MASK", "HD_ERR_BAD_ARG", "HD_ERR_OOM", "HD_ERR_CUDA", "HD_ERR_TIMEOUT",
    "HD_ERR_CANCELLED", "HD_ERR_ITER_LIMIT", "HD_ERR_NOT_READY", "HD_ERR_UNSUPPORTED", "HD_ERR_BUSY",
    "HD_SE6", "HD_SE18_FORBENCH",
]

_METRICS = {"se6": HD_SE6, "se18": HD_SE18_FORBENCH, HD_SE6: HD_SE6, HD_SE18_FORBENCH: HD_SE18_FORBENCH}


class HDError(RuntimeError):
    """A library call returned a hard error (anything but OK / EMPTY_MASK)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{N.status_string(code)} ({code}): {message}")
        self.code = code


def metric_code(metric) -> int:
    try:
        return _METRICS[metric]
    except KeyError:
        raise ValueError(f"unknown metric {metric!r}; use 'se6' or 'se18'") from None


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _dims(x):
    if len(x.shape) != 3:
        raise ValueError("masks must have shape (D, H, W)")
    D, H, W = (int(v) for v in x.shape)
    return W, H, D


_torch = None


_PAIR_DESC_DTYPE = np.dtype({
    "names": [f for f, _ in N.HdPairDesc._fields_],
    "formats": [np.uintp, np.uintp, np.int32, np.int32, np.int32, np.int32, np.int32, np.int32],
    "offsets": [getattr(N.HdPairDesc, f).offset for f, _ in N.HdPairDesc._fields_],
    "itemsize": ctypes.sizeof(N.HdPairDesc),
})


_RESULT_FIELDS = [f for f, _ in N.HdResult._fields_]
_RESULT_DTYPE = np.dtype({
    "names": _RESULT_FIELDS,
    "formats": [{ctypes.c_int32: np.int32, ctypes.c_uint64: np.uint64, ctypes.c_double: np.float64}[t]
                for _, t in N.HdResult._fields_],
    "offsets": [getattr(N.HdResult, f).offset for f in _RESULT_FIELDS],
    "itemsize": ctypes.sizeof(N.HdResult),
})


def _result_dicts(res, n):
    """hd_result array -> list of dicts, column-wise through numpy."""
    arr = np.frombuffer(res, dtype=_RESULT_DTYPE, count=n)
    cols = [arr[f].tolist() for f in _RESULT_FIELDS]
    return list(map(dict, map(zip, [_RESULT_FIELDS] * n, zip(*cols))))


class _Buf:
    """Pointer to a contiguous uint8 view of a mask (keeps the owner alive)."""

    def __init__(self, x):
        if _is_torch(x):
            import torch
            t = x
            if t.dtype != torch.uint8:
                t = (t != 0).to(torch.uint8)
            t = t.contiguous()
            self.obj = t
            self.ptr = t.data_ptr()
            self.on_device = t.is_cuda
        else:
            a = np.ascontiguousarray(x)
            if a.dtype != np.uint8:
                a = (a != 0).astype(np.uint8)
            self.obj = a
            self.ptr = a.ctypes.data
            self.on_device = False
        self.W, self.H, self.D = _dims(self.obj)


def _check(code: int, ctx_handle, allow_empty=True):
    if code == HD_OK or (allow_empty and code == HD_EMPTY_MASK):
        return
    msg = ""
    if ctx_handle:
        msg = (N.load().hd_context_last_error(ctx_handle) or b"").decode()
    raise HDError(code, msg)


RESULT_BYTES = ctypes.sizeof(N.HdResult)


def result_from_bytes(buf) -> dict:
    """hd_result from its bytes (a CPU uint8 tensor / numpy array / bytes)."""
    raw = bytes(buf.numpy().tobytes()) if hasattr(buf, "numpy") else bytes(buf)
    return N.HdResult.from_buffer_copy(raw[:RESULT_BYTES]).as_dict()


def _ready(*bufs):
    """Entry points without a stream argument run on the context's own
    stream: finish the work that produced CUDA masks on torch's stream."""
    if any(b.on_device for b in bufs):
        import torch
        torch.cuda.current_stream().synchronize()


def _current_stream_ptr():
    """torch's current stream as a cudaStream_t for the C ABI.  torch's
    default stream is the legacy NULL stream, which the C ABI would read as
    "the context's own stream": pass the cudaStreamLegacy handle (0x1)
    instead, so the work is ordered with torch's."""
    import torch
    return torch.cuda.current_stream().cuda_stream or 0x1


class Context:
    """A device context of the library (hd_context_create).

    Options mirror ``hd_options``: kernel (1 = one dilation step per grid
    barrier, 2 = temporally blocked; 0 = tuned/default), steps_per_barrier
    (kernel 2: 1 or 2), brick_x_words / brick_z (brick shape; 0 = tuned),
    ctas_per_sm (0 = occupancy maximum), max_iterations (0 = W+H+D),
    barrier_timeout_ns (0 = 10 s), percentile (robust HD, default 0.95),
    zero_copy (host masks read in place when the device can), tuning_table
    (JSON path of the autotuner's table), label (0 = nonzero voxels are
    foreground; 1..255 = voxels equal to label, the reference's
    numberToLookFor).
    """

    def __init__(self, device: int = 0, *, brick_x_words=0, brick_z=0, ctas_per_sm=0, max_iterations=0,
                 barrier_timeout_ns=0, percentile=0.95, zero_copy=True, tuning_table=None,
                 record_timings=False, kernel=0, steps_per_barrier=0, label=0):
        L = N.load()
        opt = N.HdOptions()
        L.hd_options_init(ctypes.byref(opt))
        opt.brick_x_words = brick_x_words
        opt.brick_z = brick_z
        opt.ctas_per_sm = ctas_per_sm
        opt.max_iterations = max_iterations
        opt.barrier_timeout_ns = barrier_timeout_ns
        opt.percentile = percentile
        opt.zero_copy = 1 if zero_copy else 0
        self._tuning = tuning_table.encode() if tuning_table else None
        opt.tuning_table = self._tuning
        opt.record_timings = 1 if record_timings else 0
        opt.kernel = int(kernel)
        opt.steps_per_barrier = int(steps_per_barrier)
        opt.label = int(label)
        h = ctypes.c_void_p()
        code = L.hd_context_create(int(device), ctypes.byref(opt), ctypes.byref(h))
        if code != HD_OK:
            raise HDError(code, f"hd_context_create(device={device})")
        self._h = h
        self.device = device
        self._unflushed = []  # outputs of pipelined calls not yet flushed

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            N.load().hd_context_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def last_error(self) -> str:
        return (N.load().hd_context_last_error(self._h) or b"").decode()

    def last_timings(self) -> dict:
        """Kernel durations of the last pair computation (record_timings=True)."""
        t = N.HdTimings()
        N.load().hd_context_last_timings(self._h, ctypes.byref(t))
        return t.as_dict()

    # -- single pair --------------------------------------------------------
    def compute(self, a, b, metric="se6", stream=None) -> dict:
        """HD of one pair.  Host inputs go through hd_compute_u8 (copies or
        zero-copy reads inside the call); CUDA tensors through
        hd_compute_u8_device on `stream` (default: torch's current stream)."""
        A, B = _Buf(a), _Buf(b)
        if (A.W, A.H, A.D) != (B.W, B.H, B.D):
            raise ValueError("mask shapes differ")
        if A.on_device != B.on_device:
            raise ValueError("both masks must be on the host or both on the device")
        r = N.HdResult()
        L = N.load()
        if A.on_device:
            s = _current_stream_ptr() if stream is None else stream
            code = L.hd_compute_u8_device(self._h, A.ptr, B.ptr, A.W, A.H, A.D, metric_code(metric),
                                          ctypes.c_void_p(s), ctypes.byref(r))
        else:
            code = L.hd_compute_u8(self._h, A.ptr, B.ptr, A.W, A.H, A.D, metric_code(metric), ctypes.byref(r))
        _check(code, self._h)
        return r.as_dict()

    def compute_device(self, a, b, metric="se6", stream=None) -> dict:
        return self.compute(a, b, metric, stream)

    def compute_async(self, a, b, metric="se6", out=None, stream=None):
        """Enqueues one pair on `stream` (default: torch's current stream) and
        returns at once: CUDA masks through hd_compute_u8_device_async, host
        masks (numpy / CPU tensors; pinned for a truly asynchronous copy)
        through hd_compute_u8_async, whose copy overlaps the previous pair's
        kernels.  The result lands in `out`, a CUDA uint8 tensor of
        RESULT_BYTES bytes (allocated if None), once the stream reaches it;
        decode it with result_from_bytes(out.cpu()).  Host masks must stay
        unchanged until then.  Calls on one context must stay on one stream."""
        import torch
        A, B = _Buf(a), _Buf(b)
        if (A.W, A.H, A.D) != (B.W, B.H, B.D):
            raise ValueError("mask shapes differ")
        if A.on_device != B.on_device:
            raise ValueError("both masks must be on the host or both on the device")
        if out is None:
            dev = A.obj.device if A.on_device else torch.device("cuda", self.device)
            out = torch.empty(RESULT_BYTES, dtype=torch.uint8, device=dev)
        s = _current_stream_ptr() if stream is None else stream
        L = N.load()
        fn = L.hd_compute_u8_device_async if A.on_device else L.hd_compute_u8_async
        code = fn(self._h, A.ptr, B.ptr, A.W, A.H, A.D, metric_code(metric), ctypes.c_void_p(s),
                  ctypes.c_void_p(out.data_ptr()))
        _check(code, self._h, allow_empty=False)
        return out

    def compute_pipelined(self, a, b, metric="se6", out=None, stream=None):
        """Enqueues one pair of CUDA masks through hd_compute_u8_device_pipelined
        on `stream` (default: torch's current stream) and returns at once.
        The result lands in `out` (a CUDA uint8 tensor of RESULT_BYTES bytes,
        allocated if None) once the stream reaches a later flush(); meanwhile
        the next pair's packing may run beside this pair's dilation.  The
        stream waits for the packing's reads of the masks, so they may be
        reused or freed in stream order after the call; `out` is written by
        the dilation, which the stream waits for only at flush(), so the
        context keeps a reference to it until then.  Calls on one context
        must stay on one stream."""
        import torch
        A, B = _Buf(a), _Buf(b)
        if (A.W, A.H, A.D) != (B.W, B.H, B.D):
            raise ValueError("mask shapes differ")
        if not (A.on_device and B.on_device):
            raise ValueError("compute_pipelined() takes CUDA masks")
        if out is None:
            out = torch.empty(RESULT_BYTES, dtype=torch.uint8, device=A.obj.device)
        s = _current_stream_ptr() if stream is None else stream
        code = N.load().hd_compute_u8_device_pipelined(self._h, A.ptr, B.ptr, A.W, A.H, A.D, metric_code(metric),
                                                       ctypes.c_void_p(s), ctypes.c_void_p(out.data_ptr()))
        _check(code, self._h, allow_empty=False)
        self._unflushed.append(out)
        return out

    def flush(self, stream=None):
        """hd_pipeline_flush: `stream` (default: torch's current stream)
        waits for every pipelined call so far."""
        s = _current_stream_ptr() if stream is None else stream
        _check(N.load().hd_pipeline_flush(self._h, ctypes.c_void_p(s)), self._h)
        self._unflushed = []

    # -- batches --------------------------------------------------------------
    def batch(self, pairs: Sequence, metric="se6") -> list:
        """One hd_batch_compute over [(a, b), ...] (host or CUDA masks): one
        result dict per pair, in order."""
        if len(pairs) == 0:
            return []
        return self.prepare_batch(pairs, metric).run()

    def prepare_batch(self, pairs: Sequence, metric="se6") -> "PreparedBatch":
        """The descriptor array of a batch, built once for repeated runs over
        the same mask buffers (an evaluation or serving loop that refills
        them between runs); see PreparedBatch."""
        return PreparedBatch(self, pairs, metric)

    # -- instrumentation --------------------------------------------------------
    def profile(self, a, b, metric="se6"):
        """Instrumented run (CUDA masks): result, per-step 32^3 tile counts of
        both directions (tiles_ab: dilation of B covering A) and bricks
        processed."""
        A, B = _Buf(a), _Buf(b)
        if not (A.on_device and B.on_device):
            raise ValueError("profile() takes CUDA tensors")
        n = A.W + A.H + A.D + 1
        tab = np.zeros(n, np.uint64)
        tba = np.zeros(n, np.uint64)
        bricks = ctypes.c_uint64(0)
        r = N.HdResult()
        u64p = ctypes.POINTER(ctypes.c_uint64)
        _ready(A, B)
        code = N.load().hd_profile_u8_device(self._h, A.ptr, B.ptr, A.W, A.H, A.D, metric_code(metric),
                                             ctypes.byref(r), tab.ctypes.data_as(u64p),
                                             tba.ctypes.data_as(u64p), n, ctypes.byref(bricks))
        _check(code, self._h)
        return r.as_dict(), tab, tba, int(bricks.value)

    def distance_map(self, a, b, metric="se6"):
        """Per-voxel distances (CUDA masks): int32 maps, map_a[v] = d(v, B) on
        A minus B, 0 on the overlap, -1 elsewhere (map_b likewise)."""
        import torch
        A, B = _Buf(a), _Buf(b)
        if not (A.on_device and B.on_device):
            raise ValueError("distance_map() takes CUDA tensors")
        ma = torch.empty(A.obj.shape, dtype=torch.int32, device=A.obj.device)
        mb = torch.empty(A.obj.shape, dtype=torch.int32, device=A.obj.device)
        r = N.HdResult()
        _ready(A, B)  # also orders the maps' allocation before the library writes them
        code = N.load().hd_distance_map_device(self._h, A.ptr, B.ptr, A.W, A.H, A.D, metric_code(metric),
                                               ma.data_ptr(), mb.data_ptr(), ctypes.byref(r))
        _check(code, self._h)
        return r.as_dict(), ma, mb

    def compute_hdf5(self, path_a: str, dataset_a: str, path_b: str, dataset_b: str, shape, metric="se6") -> dict:
        """The reference's HDF5 host path for one pair (hd_compute_hdf5):
        two flat boolean datasets of D*H*W elements, x fastest; shape =
        (D, H, W)."""
        D, H, W = (int(v) for v in shape)
        r = N.HdResult()
        code = N.load().hd_compute_hdf5(self._h, path_a.encode(), dataset_a.encode(), path_b.encode(),
                                        dataset_b.encode(), W, H, D, metric_code(metric), ctypes.byref(r))
        _check(code, self._h)
        return r.as_dict()

    def autotune(self, pairs: Sequence, metric="se6", repeats: int = 3) -> str:
        n = len(pairs)
        bufs = []
        descs = (N.HdPairDesc * n)()
        for i, (a, b) in enumerate(pairs):
            A, B = _Buf(a), _Buf(b)
            bufs.append((A, B))
            descs[i].a, descs[i].b = A.ptr, B.ptr
            descs[i].W, descs[i].H, descs[i].D = A.W, A.H, A.D
            descs[i].metric = metric_code(metric)
            descs[i].on_device = 1 if A.on_device else 0
        rep = ctypes.create_string_buffer(8192)
        _ready(*[x for ab in bufs for x in ab])
        code = N.load().hd_autotune(self._h, descs, n, int(repeats), rep, len(rep))
        _check(code, self._h, allow_empty=False)
        return rep.value.decode()


class PreparedBatch:
    """A batch whose descriptor array (mask pointers and sizes, filled
    column-wise through numpy) is built once; run() makes one
    hd_batch_compute call over it.  The masks must stay allocated (and
    their pointers unchanged) while the batch is in use; their contents may
    change between runs."""

    def __init__(self, ctx: "Context", pairs: Sequence, metric="se6"):
        n = len(pairs)
        keep, rows = [], []
        any_dev = False
        global _torch
        if _torch is None:
            try:
                import torch
                _torch = torch
            except ImportError:
                pass
        T = _torch.Tensor if _torch is not None else None
        u8 = _torch.uint8 if _torch is not None else None
        for i, (a, b) in enumerate(pairs):
            # contiguous 3-D uint8 CUDA tensors: a handful of attribute reads
            # inline (batches touch hundreds of tensors); anything else
            # through _Buf
            if (type(a) is T and type(b) is T and a.dtype is u8 and b.dtype is u8 and a.is_cuda and b.is_cuda
                    and a.is_contiguous() and b.is_contiguous()):
                sh = a.shape
                if len(sh) == 3 and sh == b.shape:
                    keep.append((a, b))
                    rows.append((a.data_ptr(), b.data_ptr(), sh[2], sh[1], sh[0], 1))
                    any_dev = True
                    continue
            A, B = _Buf(a), _Buf(b)
            if (A.W, A.H, A.D) != (B.W, B.H, B.D) or A.on_device != B.on_device:
                raise ValueError(f"pair {i}: shapes or devices differ")
            keep.append((A, B))
            any_dev = any_dev or A.on_device
            rows.append((A.ptr, B.ptr, A.W, A.H, A.D, 1 if A.on_device else 0))
        descs = np.zeros(n, dtype=_PAIR_DESC_DTYPE)
        if n:
            cols = np.array(rows, dtype=np.int64).T
            descs["a"], descs["b"] = cols[0], cols[1]
            descs["W"], descs["H"], descs["D"] = cols[2], cols[3], cols[4]
            descs["metric"] = metric_code(metric)
            descs["on_device"] = cols[5]
        self._ctx, self._keep, self._descs, self._n, self._dev = ctx, keep, descs, n, any_dev
        self._ptr = descs.ctypes.data_as(ctypes.POINTER(N.HdPairDesc))
        self._res = (N.HdResult * max(n, 1))()

    def __len__(self):
        return self._n

    def run(self, columns: bool = False):
        """Computes every pair.  Returns one result dict per pair, or with
        columns=True one numpy array per result field (hd, sum_ab, ...,
        avg_hd; pair i at index i), which skips building a dict per pair."""
        n = self._n
        if n == 0:
            return {f: np.zeros(0, _RESULT_DTYPE[f]) for f in _RESULT_FIELDS} if columns else []
        if self._dev:
            _torch.cuda.current_stream().synchronize()  # this call runs on the context's stream
        code = N.load().hd_batch_compute(self._ctx._h, self._ptr, n, self._res)
        _check(code, self._ctx._h)
        if columns:
            arr = np.frombuffer(self._res, dtype=_RESULT_DTYPE, count=n)
            return {f: arr[f].copy() for f in _RESULT_FIELDS}
        return _result_dicts(self._res, n)


class Server:
    """Continuous-batching request loop (hd_server_*) on a Context."""

    def __init__(self, ctx: Context, *, hbm_budget_bytes=0, max_inflight=0, max_queue=0, tick_iterations=0,
                 metric="se6"):
        L = N.load()
        opt = N.HdServerOptions()
        L.hd_server_options_init(ctypes.byref(opt))
        if hbm_budget_bytes:
            opt.hbm_budget_bytes = int(hbm_budget_bytes)
        if max_inflight:
            opt.max_inflight = int(max_inflight)
        if max_queue:
            opt.max_queue = int(max_queue)
        if tick_iterations:
            opt.tick_iterations = int(tick_iterations)
        opt.metric = metric_code(metric)
        self.metric = opt.metric
        h = ctypes.c_void_p()
        code = L.hd_server_create(ctx.handle, ctypes.byref(opt), ctypes.byref(h))
        if code != HD_OK:
            raise HDError(code, "hd_server_create")
        self._h = h
        self._ctx = ctx
        self._keep = {}

    def submit(self, a, b) -> int:
        """Queue a pair.  CUDA masks are read later on the server's own
        stream, so the work that produced them is waited for here."""
        A, B = _Buf(a), _Buf(b)
        if A.on_device or B.on_device:
            import torch
            torch.cuda.current_stream().synchronize()
        d = N.HdPairDesc()
        d.a, d.b = A.ptr, B.ptr
        d.W, d.H, d.D = A.W, A.H, A.D
        d.metric = self.metric
        d.on_device = 1 if A.on_device else 0
        t = ctypes.c_uint64(0)
        code = N.load().hd_server_submit(self._h, ctypes.byref(d), ctypes.byref(t))
        if code != HD_OK:
            raise HDError(code, "hd_server_submit")
        if A.on_device:
            self._keep[int(t.value)] = (A, B)  # device masks must outlive the request
        return int(t.value)

    def poll(self, ticket: int):
        r = N.HdResult()
        code = N.load().hd_server_poll(self._h, ticket, ctypes.byref(r))
        if code == HD_ERR_NOT_READY:
            return None
        if code != HD_OK:
            raise HDError(code, "hd_server_poll")
        self._keep.pop(ticket, None)
        return r.as_dict()

    def wait(self, ticket: int, timeout_ms: int = -1):
        r = N.HdResult()
        code = N.load().hd_server_wait(self._h, ticket, int(timeout_ms), ctypes.byref(r))
        if code == HD_ERR_NOT_READY:
            return None
        if code != HD_OK:
            raise HDError(code, "hd_server_wait")
        self._keep.pop(ticket, None)
        return r.as_dict()

    def wait_any(self, timeout_ms: int = -1):
        """(ticket, result) of the earliest finished request not yet taken,
        waiting up to timeout_ms (< 0: no limit); None on timeout."""
        r = N.HdResult()
        t = ctypes.c_uint64(0)
        code = N.load().hd_server_wait_any(self._h, int(timeout_ms), ctypes.byref(t), ctypes.byref(r))
        if code == HD_ERR_NOT_READY:
            return None
        if code != HD_OK:
            raise HDError(code, "hd_server_wait_any")
        self._keep.pop(int(t.value), None)
        return int(t.value), r.as_dict()

    def cancel(self, ticket: int):
        code = N.load().hd_server_cancel(self._h, ticket)
        if code != HD_OK:
            raise HDError(code, "hd_server_cancel")

    def stats(self) -> dict:
        s = N.HdServerStats()
        N.load().hd_server_get_stats(self._h, ctypes.byref(s))
        return s.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            N.load().hd_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Volume:
    """Mirror of the reference's Volume (forBench/Volume.h:7-26): a zeroed
    byte mask with x + W*y + W*H*z indexing."""

    def __init__(self, width: int, height: int, depth: int = 1):
        self.width, self.height, self.depth = int(width), int(height), int(depth)
        self.volume = np.zeros((self.depth, self.height, self.width), np.uint8)

    @classmethod
    def from_array(cls, arr) -> "Volume":
        a = np.ascontiguousarray(arr)
        v = cls(a.shape[2], a.shape[1], a.shape[0])
        v.volume[...] = a != 0
        return v

    def getVoxelValue(self, x, y, z) -> bool:
        return bool(self.volume[z, y, x])

    def getPixelValue(self, x, y) -> bool:
        return bool(self.volume[0, y, x])

    def setVoxelValue(self, value, x, y, z):
        self.volume[z, y, x] = 1 if value else 0

    def setPixelValue(self, value, x, y):
        self.volume[0, y, x] = 1 if value else 0

    def getWidth(self):
        return self.width

    def getHeight(self):
        return self.height

    def getDepth(self):
        return self.depth

    def getVolume(self):
        return self.volume

    def dispose(self):
        self.volume = None


class HausdorffDistance:
    """Mirror of the reference's class (forBench/HausdorffDistance.cuh:11-19).

    computeDistance(img1, img2) returns the HD as an int like the reference
    (forBench/HausdorffDistance.cu:185); the sizes of img1 are used for both
    masks (:103).  Instead of exiting the process or looping forever it
    returns -1 on error or when exactly one mask is empty.  The default element
    is the reference's shipped one (CHEBYSHEV 1 -> "se18")."""

    _ctx = None

    def __init__(self, metric="se18", device: int = 0):
        self.metric = metric_code(metric)
        self.device = device

    @classmethod
    def _context(cls, device):
        if cls._ctx is None:
            cls._ctx = Context(device)
        return cls._ctx

    def computeResult(self, img1: Volume, img2: Volume) -> dict:
        W, H, D = img1.getWidth(), img1.getHeight(), img1.getDepth()
        b = np.ascontiguousarray(img2.getVolume()).reshape(-1)[: W * H * D].reshape(D, H, W)
        return self._context(self.device).compute(img1.getVolume(), b, self.metric)

    def computeDistance(self, img1: Volume, img2: Volume) -> int:
        try:
            r = self.computeResult(img1, img2)
        except HDError:
            return -1
        return int(r["hd"]) if r["status"] == HD_OK else -1

    def computeDistances(self, img1: Volume, img2: Volume):
        """(max HD, average HD), (-1, -1.0) on error."""
        try:
            r = self.computeResult(img1, img2)
        except HDError:
            return -1, -1.0
        if r["status"] != HD_OK:
            return -1, -1.0
        return int(r["hd"]), float(r["avg_hd"])


def load_hdf5_bool(path: str, dataset: str) -> np.ndarray:
    """loadHDFIntoBoolArr (forBench/hdf5Manag.cu:44-86): flat uint8 array."""
    L = N.load()
    p = ctypes.c_void_p()
    n = ctypes.c_size_t(0)
    code = L.hd_load_hdf5_bool(path.encode(), dataset.encode(), ctypes.byref(p), ctypes.byref(n))
    if code != HD_OK:
        raise HDError(code, f"hd_load_hdf5_bool({path!r}, {dataset!r})")
    try:
        return np.ctypeslib.as_array((ctypes.c_uint8 * n.value).from_address(p.value)).copy()
    finally:
        L.hd_free(p)
