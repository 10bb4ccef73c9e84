"""Python host binding of liblsb.so, the GB300 LSD radix-sort pass library.

The library's C ABI (include/lsb.h) is the drop-in boundary for the sort loop
of mpi/mpi_lsbsort.cpp (mppf/distributed-lsb): ``sort_pairs`` is ``mySort``
(mpi/mpi_lsbsort.cpp:592-597), ``global_shuffle`` is one ``globalShuffle``
pass (:493-589) and ``histogram`` is the count loop of ``localShuffle``
(:237-241) for every digit. This module only loads the shared library and
passes device pointers through ctypes; PyTorch supplies device memory and
streams. There is no fallback: if liblsb.so is missing or fails to load, every
call raises.

Arrays are int64 CUDA tensors of shape (n, 2) -- column 0 the key, column 1
the value, bit-for-bit the reference's 16-byte ``SortElement``; view them as
uint64 on the host (``t.cpu().numpy().view(numpy.uint64)``).
"""
from __future__ import annotations

import ctypes
import os

from ._build import LIB_PATH, build, lib_path  # noqa: F401

LSB_OK = 0
LSB_ERR_INVALID_ARG = 1
LSB_ERR_ALIGNMENT = 2
LSB_ERR_TOO_LARGE = 3
LSB_ERR_WORKSPACE = 4
LSB_ERR_CUDA = 5
LSB_ERR_DEVICE_TIMEOUT = 6
LSB_ERR_NO_DEVICE = 7
LSB_ERR_OVERLAP = 8
LSB_ERR_NO_MEMORY = 9

DIST_UNIFORM, DIST_LOW32, DIST_ZIPF, DIST_EQUAL, DIST_NEARLY_SORTED = 0, 1, 2, 3, 4
DIST_NAMES = {"uniform": 0, "low32": 1, "zipf": 2, "equal": 3, "nearly_sorted": 4}

# Every symbol include/lsb.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
SIGNATURES = {
    "lsb_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "lsb_version": (ctypes.c_int, []),
    "lsb_num_passes": (ctypes.c_int, [ctypes.c_int]),
    "lsb_workspace_bytes": (ctypes.c_int, [_I64, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    "lsb_sort_pairs": (ctypes.c_int, [_P, _P, _I64, ctypes.c_int, _P, ctypes.c_size_t, _P]),
    "lsb_pass": (ctypes.c_int, [_P, _P, _I64, ctypes.c_int, ctypes.c_int, _P, ctypes.c_size_t, _P]),
    "lsb_pass_workspace_bytes": (ctypes.c_int, [_I64, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    "lsb_histogram": (ctypes.c_int, [_P, _I64, ctypes.c_int, _P, _P]),
    "lsb_query": (ctypes.c_int, [_P, _P, _P]),
    "lsb_sort_pairs_host": (ctypes.c_int, [_P, _I64, ctypes.c_int, _P]),
    "lsb_generate": (ctypes.c_int, [_P, _I64, ctypes.c_int, ctypes.c_uint64, _P]),
    "lsb_verify": (ctypes.c_int, [_P, _P, _I64, ctypes.POINTER(ctypes.c_uint64), _P]),
    "lsb_sort_pairs_noalloc": (ctypes.c_int, [_P, _P, _I64, ctypes.c_int, _P]),
    "lsb_segmented_workspace_bytes": (ctypes.c_int, [_I64, _I64, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    "lsb_sort_segmented": (ctypes.c_int, [_P, _P, _I64, _P, _I64, _P, _P, ctypes.c_size_t, _P]),
    "lsb_tune_segmented": (ctypes.c_int, [_P, _I64, _P, _P]),
    "lsb_graph_capture_segmented": (ctypes.c_int, [_P, _P, _I64, _P, _I64, _P, _P, ctypes.c_size_t,
                                                   ctypes.POINTER(ctypes.c_void_p)]),
    "lsb_graph_launch": (ctypes.c_int, [_P, _P]),
    "lsb_graph_destroy": (ctypes.c_int, [_P]),
    "lsb_server_create": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_void_p)]),
    "lsb_server_submit_host": (ctypes.c_int, [_P, _P, _I64, ctypes.POINTER(ctypes.c_uint64)]),
    "lsb_server_submit_generated": (ctypes.c_int, [_P, _I64, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                                   ctypes.POINTER(ctypes.c_uint64)]),
    "lsb_server_wait": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.c_double, _P]),
    "lsb_server_fetch": (ctypes.c_int, [_P, ctypes.c_uint64, _P, _I64]),
    "lsb_server_stats": (ctypes.c_int, [_P, _P]),
    "lsb_server_device_stats": (ctypes.c_int, [_P, _P]),
    "lsb_server_destroy": (ctypes.c_int, [_P]),
    "lsb_profile_enable": (ctypes.c_int, [ctypes.c_int]),
    "lsb_profile_read": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "lsb_selftest_wait_timeout": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    "lsb_selftest_wait": (ctypes.c_int, [ctypes.c_int, _P, ctypes.POINTER(ctypes.c_int)]),
    "lsb_exchange_plan": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _I64, ctypes.c_int, _P, _P, _P, _P, _P,
                                         ctypes.POINTER(ctypes.c_int64)]),
    "lsb_place_pieces": (ctypes.c_int, [_P, _I64, _P, _I64, _P, _P, _P, _I64, _P]),
}


class KernelTime(ctypes.Structure):
    """lsb_kernel_time_t"""

    _fields_ = [("name", ctypes.c_char * 40), ("launches", ctypes.c_int64), ("total_ms", ctypes.c_double)]


class Tuning(ctypes.Structure):
    """lsb_tuning_t"""

    _fields_ = [("digit_bits", ctypes.c_int32), ("variant", ctypes.c_int32), ("ctas", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class ServerConfig(ctypes.Structure):
    """lsb_server_config_t"""

    _fields_ = [("slots", ctypes.c_int32), ("digit_bits", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64),
                ("batch_max_elems", ctypes.c_int64), ("batch_max_requests", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class RequestInfo(ctypes.Structure):
    """lsb_request_info_t"""

    _fields_ = [("status", ctypes.c_int32), ("batch", ctypes.c_int32), ("n", ctypes.c_int64),
                ("latency_ms", ctypes.c_double), ("queue_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    """lsb_server_stats_t"""

    _fields_ = [("requests_done", ctypes.c_int64), ("elements_done", ctypes.c_int64), ("units", ctypes.c_int64),
                ("batched_requests", ctypes.c_int64), ("peak_bytes", ctypes.c_int64),
                ("budget_bytes", ctypes.c_int64), ("latency_p50_ms", ctypes.c_double),
                ("latency_p99_ms", ctypes.c_double), ("service_p50_ms", ctypes.c_double),
                ("service_p99_ms", ctypes.c_double), ("wall_ms", ctypes.c_double),
                ("elements_per_s", ctypes.c_double)]


class Stats(ctypes.Structure):
    """lsb_stats_t"""

    _fields_ = [
        ("device_status", ctypes.c_int32),
        ("passes_planned", ctypes.c_int32),
        ("passes_run", ctypes.c_int32),
        ("skipped_mask", ctypes.c_uint32),
        ("final_copy", ctypes.c_int32),
        ("digit_bits", ctypes.c_int32),
        ("n", ctypes.c_int64),
    ]


class LsbError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} ({status})")


_lib = None


def load(path: str | None = None):
    """Load liblsb.so (once). Raises if it is missing: there is no fallback."""
    global _lib
    if _lib is None:
        p = path or lib_path()
        if not os.path.exists(p):
            raise FileNotFoundError(f"liblsb.so not built ({p}); run build() first")
        L = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def status_string(status: int) -> str:
    try:
        return load().lsb_status_string(status).decode()
    except Exception:  # pragma: no cover - only for messages
        return str(status)


def _check(rc: int, what: str) -> None:
    if rc != LSB_OK:
        raise LsbError(rc, what)


def _stream_ptr(stream):
    if stream is None:
        import torch

        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _ptr(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() else ctypes.c_void_p(0)


def num_passes(digit_bits: int) -> int:
    return load().lsb_num_passes(digit_bits)


def workspace_bytes(n: int, digit_bits: int) -> int:
    out = ctypes.c_size_t(0)
    _check(load().lsb_workspace_bytes(n, digit_bits, ctypes.byref(out)), "lsb_workspace_bytes")
    return out.value


def alloc_workspace(n: int, digit_bits: int, device=None):
    import torch

    nbytes = workspace_bytes(n, digit_bits)
    return torch.empty(max(nbytes, 256), dtype=torch.uint8, device=device or "cuda")


def sort_pairs(a, b, digit_bits: int = 16, workspace=None, stream=None) -> None:
    """mySort(A, B): sorts ``a`` (int64 (n, 2) CUDA tensor) in place by key,
    stably; ``b`` is scratch of the same shape. Asynchronous when a workspace
    tensor is given, blocking (and status-checked) otherwise."""
    n = a.shape[0]
    ws = _ptr(workspace) if workspace is not None else ctypes.c_void_p(0)
    wsb = workspace.numel() if workspace is not None else 0
    _check(load().lsb_sort_pairs(_ptr(a), _ptr(b), n, digit_bits, ws, wsb, _stream_ptr(stream)),
           "lsb_sort_pairs")


def pass_workspace_bytes(n: int, digit_bits: int) -> int:
    """Workspace of lsb_pass at its fastest (scratch for wide-digit sub-passes)."""
    out = ctypes.c_size_t(0)
    _check(load().lsb_pass_workspace_bytes(n, digit_bits, ctypes.byref(out)), "lsb_pass_workspace_bytes")
    return out.value


def global_shuffle(src, dst, digit: int, digit_bits: int = 16, workspace=None, stream=None) -> None:
    """One pass: ``dst`` = ``src`` stably sorted by ``digit``."""
    n = src.shape[0]
    ws = _ptr(workspace) if workspace is not None else ctypes.c_void_p(0)
    wsb = workspace.numel() if workspace is not None else 0
    _check(load().lsb_pass(_ptr(src), _ptr(dst), n, digit_bits, digit, ws, wsb, _stream_ptr(stream)),
           "lsb_pass")


def histogram(data, digit_bits: int = 16, stream=None):
    """Counts of every digit of every pass: int64 CUDA tensor [passes, 2^b]."""
    import torch

    p = num_passes(digit_bits)
    out = torch.empty((p, 1 << digit_bits), dtype=torch.int64, device=data.device)
    _check(load().lsb_histogram(_ptr(data), data.shape[0], digit_bits, _ptr(out), _stream_ptr(stream)),
           "lsb_histogram")
    return out


def exchange_plan(counts, n: int, rank: int):
    """lsb_exchange_plan: the exchange of one pass of the sharded sort for
    `rank` from the all-gathered count table counts[R][2^b] (int64 numpy).
    Returns (send_counts, recv_counts, piece_src, piece_dst, piece_len), all
    int64 numpy arrays (host computation, no GPU needed)."""
    import numpy as np

    c = np.ascontiguousarray(counts, dtype=np.int64)
    ranks, nbins = c.shape
    bits = nbins.bit_length() - 1
    if nbins != 1 << bits:
        raise ValueError("count table width must be a power of two")
    send = np.zeros(ranks, np.int64)
    recv = np.zeros(ranks, np.int64)
    cap = max(1, ranks * nbins)
    src, dst, ln = (np.zeros(cap, np.int64) for _ in range(3))
    npieces = ctypes.c_int64(0)
    ptr = lambda a: ctypes.c_void_p(a.ctypes.data)
    _check(load().lsb_exchange_plan(ptr(c), ranks, bits, n, rank, ptr(send), ptr(recv), ptr(src), ptr(dst),
                                    ptr(ln), ctypes.byref(npieces)), "lsb_exchange_plan")
    k = npieces.value
    return send, recv, src[:k].copy(), dst[:k].copy(), ln[:k].copy()


def place_pieces(received, out, piece_src, piece_dst, piece_len, stream=None) -> None:
    """lsb_place_pieces: out[piece_dst[i] .. + piece_len[i]) = received[piece_src[i] ..]
    (CUDA int64 (m, 2) tensors; piece tables int64 numpy arrays)."""
    import numpy as np

    tabs = [np.ascontiguousarray(t, dtype=np.int64) for t in (piece_src, piece_dst, piece_len)]
    ptrs = [ctypes.c_void_p(t.ctypes.data) for t in tabs]
    _check(load().lsb_place_pieces(_ptr(received), received.shape[0], _ptr(out), out.shape[0], *ptrs,
                                   len(tabs[0]), _stream_ptr(stream)), "lsb_place_pieces")


def query(workspace, stream=None) -> Stats:
    s = Stats()
    load().lsb_query(_ptr(workspace), _stream_ptr(stream), ctypes.byref(s))
    return s


def sort_pairs_host(array, digit_bits: int = 16) -> None:
    """Host-memory mySort on a numpy uint64 (n, 2) array or a CPU tensor, in
    place: copy in, sort, copy out (blocking)."""
    if hasattr(array, "data_ptr"):
        ptr, n = array.data_ptr(), array.shape[0]
    else:
        ptr, n = array.ctypes.data, array.shape[0]
    _check(load().lsb_sort_pairs_host(ctypes.c_void_p(ptr), n, digit_bits, _stream_ptr(None)),
           "lsb_sort_pairs_host")


def generate(n: int, dist: int = DIST_UNIFORM, seed: int = 1, out=None, device=None, stream=None):
    import torch

    if out is None:
        out = torch.empty((n, 2), dtype=torch.int64, device=device or "cuda")
    _check(load().lsb_generate(_ptr(out), n, dist, seed, _stream_ptr(stream)), "lsb_generate")
    return out


def segmented_workspace_bytes(n_total: int, nseg: int, digit_bits: int = 16) -> int:
    out = ctypes.c_size_t(0)
    _check(load().lsb_segmented_workspace_bytes(n_total, nseg, digit_bits, ctypes.byref(out)),
           "lsb_segmented_workspace_bytes")
    return out.value


def alloc_segmented_workspace(n_total: int, nseg: int, digit_bits: int = 16, device=None):
    import torch

    nbytes = segmented_workspace_bytes(n_total, nseg, digit_bits)
    return torch.empty(max(nbytes, 256), dtype=torch.uint8, device=device or "cuda")


def tune_segmented(offsets_host, stream=None) -> Tuning:
    """The autotuner: best (digit width, kernel shape) for this size mix."""
    import numpy as np

    off = np.ascontiguousarray(offsets_host, dtype=np.int64)
    t = Tuning()
    _check(load().lsb_tune_segmented(ctypes.c_void_p(off.ctypes.data), off.shape[0] - 1, ctypes.byref(t),
                                     _stream_ptr(stream)), "lsb_tune_segmented")
    return t


def sort_segmented(a, b, offsets, tuning: Tuning | None = None, workspace=None, stream=None) -> None:
    """Sorts every segment a[offsets[s]:offsets[s+1]] in place (offsets: int64
    CUDA tensor of nseg + 1 entries)."""
    ws = _ptr(workspace) if workspace is not None else ctypes.c_void_p(0)
    wsb = workspace.numel() if workspace is not None else 0
    tp = ctypes.byref(tuning) if tuning is not None else None
    _check(load().lsb_sort_segmented(_ptr(a), _ptr(b), a.shape[0], _ptr(offsets), offsets.shape[0] - 1, tp,
                                     ws, wsb, _stream_ptr(stream)), "lsb_sort_segmented")


class SegmentedGraph:
    """The batch sort captured into a CUDA graph (lsb_graph_capture_segmented)."""

    def __init__(self, a, b, offsets, tuning: Tuning | None, workspace):
        self._keep = (a, b, offsets, workspace)
        h = ctypes.c_void_p(0)
        tp = ctypes.byref(tuning) if tuning is not None else None
        _check(load().lsb_graph_capture_segmented(_ptr(a), _ptr(b), a.shape[0], _ptr(offsets),
                                                  offsets.shape[0] - 1, tp, _ptr(workspace),
                                                  workspace.numel(), ctypes.byref(h)),
               "lsb_graph_capture_segmented")
        self.handle = h

    def launch(self, stream=None) -> None:
        _check(load().lsb_graph_launch(self.handle, _stream_ptr(stream)), "lsb_graph_launch")

    def close(self) -> None:
        if self.handle:
            load().lsb_graph_destroy(self.handle)
            self.handle = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ServerDeviceStats(ctypes.Structure):
    """lsb_server_device_stats_t"""

    _fields_ = [("units_timed", ctypes.c_int64), ("busy_ms", ctypes.c_double), ("unit_ms_sum", ctypes.c_double),
                ("overlap", ctypes.c_double), ("max_concurrent", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Server:
    """The request loop (lsb_server_*): continuous batching of sort requests."""

    def __init__(self, slots: int = 4, digit_bits: int = 16, hbm_budget_bytes: int = 0,
                 batch_max_elems: int = 0, batch_max_requests: int = 0):
        cfg = ServerConfig(slots=slots, digit_bits=digit_bits, hbm_budget_bytes=hbm_budget_bytes,
                           batch_max_elems=batch_max_elems, batch_max_requests=batch_max_requests)
        h = ctypes.c_void_p(0)
        _check(load().lsb_server_create(ctypes.byref(cfg), ctypes.byref(h)), "lsb_server_create")
        self.handle = h

    def submit_generated(self, n: int, dist: int = DIST_UNIFORM, seed: int = 1, keep: bool = False) -> int:
        rid = ctypes.c_uint64(0)
        _check(load().lsb_server_submit_generated(self.handle, n, dist, seed, 1 if keep else 0, ctypes.byref(rid)),
               "lsb_server_submit_generated")
        return rid.value

    def submit_host(self, array) -> int:
        """array: numpy uint64 (n, 2) or CPU tensor; sorted in place."""
        ptr = array.data_ptr() if hasattr(array, "data_ptr") else array.ctypes.data
        rid = ctypes.c_uint64(0)
        _check(load().lsb_server_submit_host(self.handle, ctypes.c_void_p(ptr), array.shape[0], ctypes.byref(rid)),
               "lsb_server_submit_host")
        return rid.value

    def wait(self, rid: int, timeout_s: float = 600.0) -> RequestInfo:
        info = RequestInfo()
        _check(load().lsb_server_wait(self.handle, rid, timeout_s, ctypes.byref(info)), "lsb_server_wait")
        return info

    def fetch(self, rid: int, n: int):
        import numpy as np

        out = np.empty((n, 2), dtype=np.uint64)
        _check(load().lsb_server_fetch(self.handle, rid, ctypes.c_void_p(out.ctypes.data), n), "lsb_server_fetch")
        return out

    def stats(self) -> ServerStats:
        st = ServerStats()
        _check(load().lsb_server_stats(self.handle, ctypes.byref(st)), "lsb_server_stats")
        return st

    def device_stats(self) -> ServerDeviceStats:
        st = ServerDeviceStats()
        _check(load().lsb_server_device_stats(self.handle, ctypes.byref(st)), "lsb_server_device_stats")
        return st

    def close(self) -> None:
        if self.handle:
            load().lsb_server_destroy(self.handle)
            self.handle = ctypes.c_void_p(0)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def profile_enable(on: bool = True) -> None:
    _check(load().lsb_profile_enable(1 if on else 0), "lsb_profile_enable")


def profile_read() -> dict:
    """{kernel name: (launches, total device ms)} since the last read."""
    arr = (KernelTime * 64)()
    cnt = ctypes.c_int(0)
    _check(load().lsb_profile_read(ctypes.cast(arr, ctypes.c_void_p), 64, ctypes.byref(cnt)), "lsb_profile_read")
    return {arr[i].name.decode(): (arr[i].launches, arr[i].total_ms) for i in range(cnt.value)}


def selftest_wait_timeout(stream=None) -> int:
    """Runs the sort kernels' look-back wait on a predecessor that never
    publishes; returns the device status it ended with (LSB_ERR_DEVICE_TIMEOUT
    when the bounded wait ran out as designed). Takes about a second."""
    st = ctypes.c_int(-1)
    _check(load().lsb_selftest_wait_timeout(_stream_ptr(stream), ctypes.byref(st)),
           "lsb_selftest_wait_timeout")
    return st.value


WAIT_LOOKBACK, WAIT_RING_SLOT, WAIT_BULK_COPY = 0, 1, 2
WAIT_BUCKET_PREFIX, WAIT_BUCKET_LOOKBACK, WAIT_SCHEDULER = 3, 4, 5
WAITS = {"lookback": 0, "ring_slot": 1, "bulk_copy": 2, "bucket_prefix": 3, "bucket_lookback": 4,
         "scheduler": 5}


def selftest_wait(which: int, stream=None) -> int:
    """Runs one bounded device wait of the library's kernels (WAIT_*) on a
    flag nothing sets; returns the device status it ended with
    (LSB_ERR_DEVICE_TIMEOUT when the wait ran out as designed)."""
    st = ctypes.c_int(-1)
    _check(load().lsb_selftest_wait(which, _stream_ptr(stream), ctypes.byref(st)), "lsb_selftest_wait")
    return st.value


def verify(inp, out, stream=None) -> int:
    """Number of violations of "out is the stable sort by key of inp"
    (0 = identical to the reference's std::stable_sort check)."""
    bad = ctypes.c_uint64(0)
    _check(load().lsb_verify(_ptr(inp), _ptr(out), inp.shape[0], ctypes.byref(bad), _stream_ptr(stream)),
           "lsb_verify")
    return bad.value
