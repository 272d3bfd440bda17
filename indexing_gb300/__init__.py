"""GB300 WAH bitmap index builder.

Python face of the C ABI in ``include/wah/wah.h`` (library
``libwah_gb300.so``).  It mirrors the reference's phase interface
(src/phases.cpp, src/cpu.cpp):

* :func:`build_index`        whole pipeline (sort_rids_by_value ..
                             compute_colum_length) on a device column
* :func:`sort_rids_by_value` phase a1 alone
* :func:`build_sorted`       phases a2..a6 on a sorted (value, rid) stream
* :class:`HostContext`       host buffers in, host buffers out (the
                             reference's global_argument -> phases ->
                             mem_ref::data flow)
* :func:`decoded_bitmap`     one key's words as a '0'/'1' string
                             (src/cpu.cpp:47-74)
* :func:`decode`             every key's rows on the GPU (row ids, the
                             sorted column, the column itself)
* :func:`append`             the index of more rows appended to an index on
                             the GPU (incremental builds)
* :func:`parse_text`         the reference's text data files (one value per
                             line) parsed on the GPU into a column
* :func:`query`              rows of a key / value range, or of two ranges
                             combined (OR, AND, AND NOT), as row ids and as
                             a WAH bitmap

Device memory comes from torch (plumbing only); every computation runs in
the CUDA kernels of the native library.  There is no CPU fallback: without
the library or a GPU these functions raise.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import wah_counts

__all__ = ["WahError", "WahIndex", "build_index", "sort_rids_by_value", "build_sorted",
           "HostContext", "Pipeline", "Batch", "Server", "decoded_bitmap", "workspace_bytes", "output_caps",
           "MAX_ROWS", "last_launch_count", "autotune", "autotune_workload", "decode", "query",
           "parse_text", "append", "QUERY_KEYS", "QUERY_OR", "QUERY_AND", "QUERY_ANDNOT",
           "TUNE_MATCH", "TUNE_HYBRID", "TUNE_PACK", "WORKLOAD_UNIFORM", "WORKLOAD_SKEWED",
           "WORKLOAD_BATCH"]

MAX_ROWS = 1 << 31

WAH_OK, WAH_EINVAL, WAH_ENOMEM, WAH_ECUDA, WAH_ETIMEOUT, WAH_ERANGE, WAH_EOVERFLOW, \
    WAH_ENODEV, WAH_ECORRUPT = range(9)
QUERY_KEYS, QUERY_OR, QUERY_AND, QUERY_ANDNOT = range(4)
# tuning word flags (include/wah/wah.h) and autotuner workloads
TUNE_MATCH, TUNE_HYBRID, TUNE_PACK = 0x100, 0x200, 0x400
WORKLOAD_UNIFORM, WORKLOAD_SKEWED, WORKLOAD_BATCH = range(3)


def tune_later(shape: int) -> int:
    """The tile shape of the digit passes after the first, in a tuning word."""
    return shape << 16


class WahError(RuntimeError):
    """A non-zero status from the native library."""

    def __init__(self, status: int, where: str = ""):
        self.status = int(status)
        msg = _lib.load().wah_strerror(self.status).decode()
        super().__init__(f"{where}: {msg} (status {self.status})" if where else msg)


def _check(rc: int, where: str) -> None:
    if rc != WAH_OK:
        raise WahError(rc, where)


@dataclass
class WahIndex:
    """keys[K], offsets[K], index[L] plus the merged-entry count k."""
    keys: object
    offsets: object
    index: object
    merged: int

    @property
    def keycnt(self) -> int:
        return len(self.keys)

    @property
    def index_len(self) -> int:
        return len(self.index)

    def bitmap(self, i: int):
        """Words of the i-th key (src/cpu.cpp:332-335)."""
        end = int(self.offsets[i + 1]) if i + 1 < len(self.offsets) else len(self.index)
        return self.index[int(self.offsets[i]):end]

    def numpy(self) -> "WahIndex":
        def cv(a):
            return a.cpu().numpy().view(np.uint32) if hasattr(a, "cpu") else a
        return WahIndex(cv(self.keys), cv(self.offsets), cv(self.index), self.merged)


def output_caps(n: int, bound: int = 0):
    kc, ic = ctypes.c_uint64(), ctypes.c_uint64()
    _lib.load().wah_output_caps(n, bound, ctypes.byref(kc), ctypes.byref(ic))
    return kc.value, ic.value


def workspace_bytes(n: int, bound: int = 0) -> int:
    return int(_lib.load().wah_workspace_bytes(n, bound))


def last_launch_count() -> int:
    """Kernels enqueued by the last native call on this thread."""
    return int(_lib.load().wah_last_launch_count())


def _torch():
    import torch
    return torch


def autotune(n: int, bound: int = 0, cache_path: str | None = None):
    """Times every radix tile shape on a synthetic column of n rows (values
    up to bound), applies the fastest process-wide, and caches the choice per
    (device, size bucket, digit passes) in ``cache_path``.  Returns
    ``(tuning, from_cache)``."""
    lib = _lib.load()
    chosen, cached = ctypes.c_int(), ctypes.c_int()
    rc = lib.wah_autotune(n, bound, cache_path.encode() if cache_path else None,
                          ctypes.byref(chosen), ctypes.byref(cached))
    _check(rc, "wah_autotune")
    return chosen.value, bool(cached.value)


def autotune_workload(workload: int, n: int, bound: int = 0, ncols: int = 0,
                      cache_path: str | None = None):
    """Times the tile shapes on synthetic data of one workload (one uniform
    column, one skewed column, or a batch of ``ncols`` columns of about ``n``
    rows in all) and returns ``(tuning, from_cache)`` without applying it:
    pass the word to :func:`build_index`, :class:`Batch` or :class:`Server`."""
    lib = _lib.load()
    chosen, cached = ctypes.c_int(), ctypes.c_int()
    rc = lib.wah_autotune_workload(workload, n, bound, ncols,
                                   cache_path.encode() if cache_path else None,
                                   ctypes.byref(chosen), ctypes.byref(cached))
    _check(rc, "wah_autotune_workload")
    return chosen.value, bool(cached.value)


def _stream_handle(stream) -> int:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _as_device_u32(values, device):
    """uint32 data as a contiguous int32 CUDA tensor (same bits)."""
    torch = _torch()
    if isinstance(values, np.ndarray):
        arr = np.ascontiguousarray(values, dtype=np.uint32).view(np.int32)
        return torch.from_numpy(arr).to(device)
    t = values
    if t.dtype not in (torch.int32, torch.uint32):
        raise TypeError("values must be a 32-bit integer tensor")
    if t.dtype == torch.uint32:
        t = t.view(torch.int32)
    t = t.to(device).contiguous()
    if t.data_ptr() % 16:  # a view into a larger tensor: the kernels want 16-byte alignment
        t = t.clone()
    return t


class _Buffers:
    """Device outputs + workspace for one column (reusable)."""

    def __init__(self, n: int, bound: int, device):
        torch = _torch()
        kc, ic = output_caps(max(n, 1), bound)
        self.keys = torch.empty(kc, dtype=torch.int32, device=device)
        self.offsets = torch.empty(kc, dtype=torch.int32, device=device)
        self.index = torch.empty(ic, dtype=torch.int32, device=device)
        self.counts = torch.zeros(4, dtype=torch.int32, device=device)
        self.ws_bytes = workspace_bytes(max(n, 1), bound)
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=device)


def build_index(values, bound: int = 0, stream=None, device="cuda", sync: bool = True,
                buffers: _Buffers | None = None, tuning: int = 0) -> WahIndex:
    """Builds the WAH index of one uint32 column on the GPU.

    ``values``: numpy uint32 array or 32-bit integer tensor.  ``bound``: the
    largest value (the reference's ``-b``), 0 = unknown.  Returns a
    :class:`WahIndex` of CUDA int32 tensors holding uint32 bits (use
    ``.numpy()`` for numpy uint32).  With ``sync=False`` the counters are not
    read back and the full-capacity buffers are returned in a tuple instead.
    ``tuning``: this build's tile shapes (a tuning word), 0 = the process
    default.
    """
    lib = _lib.load()
    torch = _torch()
    v = _as_device_u32(values, device)
    n = v.numel()
    if n >= MAX_ROWS:
        raise WahError(WAH_ERANGE, "build_index")
    b = buffers or _Buffers(n, bound, v.device)
    rc = lib.wah_build_tuned(v.data_ptr(), n, bound, b.keys.data_ptr(), b.offsets.data_ptr(),
                             b.index.data_ptr(), b.counts.data_ptr(), b.ws.data_ptr(),
                             b.ws_bytes, tuning, _stream_handle(stream))
    _check(rc, "wah_build")
    if not sync:
        return b
    c = b.counts.cpu().numpy().view(np.uint32)
    if c[3] != WAH_OK:
        raise WahError(int(c[3]), "wah_build (device)")
    K, L, k = int(c[0]), int(c[1]), int(c[2])
    return WahIndex(b.keys[:K], b.offsets[:K], b.index[:L], k)


def _index_tensors(idx: WahIndex):
    torch = _torch()
    parts = []
    for a in (idx.keys, idx.offsets, idx.index):
        t = _as_device_u32(a, "cuda") if isinstance(a, np.ndarray) else a
        parts.append(t.contiguous())
    dev = parts[2].device if parts[2].numel() else parts[0].device
    # empty tensors may have no storage: give the kernels a valid pointer
    parts = [t if t.numel() else torch.zeros(4, dtype=torch.int32, device=dev) for t in parts]
    return parts[0], parts[1], parts[2], dev


def decode(idx: WahIndex, n: int, rows: bool = True, values: bool = False,
           column: bool = False, key_rows: bool = False, stream=None) -> dict:
    """Decodes every key of ``idx`` (an index of ``n`` rows) on the GPU.

    Returns a dict of CUDA int32 tensors (uint32 bits) for the outputs asked
    for: ``rows`` (row ids, keys ascending, rows ascending per key),
    ``values`` (the key of each of those rows), ``column`` (the column:
    ``column[row]`` = its value; rows no key covers keep 0xFFFFFFFF) and
    ``key_rows`` (position of each key's first row).  Raises WahError with
    WAH_ECORRUPT when the words do not describe exactly n rows."""
    lib = _lib.load()
    torch = _torch()
    keys, offsets, index, dev = _index_tensors(idx)
    K, L = len(idx.keys), len(idx.index)
    out = {}

    def alloc(name, size, fill=None):
        t = torch.empty(max(size, 1), dtype=torch.int32, device=dev)
        if fill is not None:
            t.fill_(fill)
        out[name] = t
        return t.data_ptr()

    p_rows = alloc("rows", n) if rows else None
    p_vals = alloc("values", n) if values else None
    p_col = alloc("column", n, -1) if column else None
    p_kr = alloc("key_rows", K) if key_rows else None
    status = torch.zeros(4, dtype=torch.int32, device=dev)
    wsb = int(lib.wah_decode_workspace_bytes())
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    rc = lib.wah_decode(keys.data_ptr(), offsets.data_ptr(), index.data_ptr(), K, L, n, p_rows,
                        p_vals, p_col, p_kr, status.data_ptr(), ws.data_ptr(), wsb,
                        _stream_handle(stream))
    _check(rc, "wah_decode")
    st = int(status[0].item())
    if st != WAH_OK:
        raise WahError(st, "wah_decode (device)")
    sizes = {"rows": n, "values": n, "column": n, "key_rows": K}
    return {k: v[:sizes[k]] for k, v in out.items()}


class _ParseResult(ctypes.Structure):
    _fields_ = [("values", ctypes.c_uint64), ("tokens", ctypes.c_uint64),
                ("max_value", ctypes.c_uint32), ("status", ctypes.c_uint32),
                ("reserved", ctypes.c_uint64)]


def parse_text(data, capacity: int | None = None, stream=None, device="cuda"):
    """Parses a text data file's bytes (one value per line, or any
    whitespace between values) on the GPU.

    ``data``: bytes, a numpy uint8 array or a uint8 tensor.  Returns
    ``(values, info)``: a CUDA int32 tensor (uint32 bits) of the values
    before the first token that is not a 32-bit decimal number, and a dict
    with ``values``, ``tokens`` and ``max_value``.  ``capacity`` bounds the
    values stored (default: one per two bytes, always enough)."""
    lib = _lib.load()
    torch = _torch()
    if isinstance(data, (bytes, bytearray, memoryview)):
        data = np.frombuffer(bytes(data), dtype=np.uint8)
    if isinstance(data, np.ndarray):
        arr = np.ascontiguousarray(data, dtype=np.uint8)
        if not arr.flags.writeable:
            arr = arr.copy()
        t = torch.from_numpy(arr).to(device)
    else:
        t = data.to(device).contiguous()
    nbytes = t.numel()
    cap = (nbytes + 1) // 2 if capacity is None else int(capacity)
    out = torch.empty(max(cap, 1), dtype=torch.int32, device=t.device)
    res = torch.zeros(4, dtype=torch.int64, device=t.device)
    wsb = int(lib.wah_parse_workspace_bytes())
    ws = torch.empty(wsb, dtype=torch.uint8, device=t.device)
    text_ptr = t.data_ptr() if nbytes else ws.data_ptr()
    rc = lib.wah_parse_text(text_ptr, nbytes, out.data_ptr(), cap, res.data_ptr(),
                            ws.data_ptr(), wsb, _stream_handle(stream))
    _check(rc, "wah_parse_text")
    r = _ParseResult.from_buffer_copy(res.cpu().numpy().tobytes())
    if r.status != WAH_OK:
        raise WahError(int(r.status), "wah_parse_text (device)")
    info = {"values": int(r.values), "tokens": int(r.tokens), "max_value": int(r.max_value)}
    return out[:int(r.values)], info


def append(a: WahIndex, rows_a: int, b: WahIndex, stream=None) -> WahIndex:
    """The index of rows_a + n rows from ``a`` (rows [0, rows_a); rows_a a
    multiple of 31) and ``b`` (the next n rows, built alone), on the GPU;
    word for word the index one build of all rows gives.  ``merged`` of the
    result is 0 (not tracked)."""
    lib = _lib.load()
    torch = _torch()
    ak, ao, ai, dev = _index_tensors(a)
    bk, bo, bi, _ = _index_tensors(b)
    ka, la, kb, lb = len(a.keys), len(a.index), len(b.keys), len(b.index)
    kc, ic = ka + kb, la + lb + kb
    out_k = torch.empty(max(kc, 1), dtype=torch.int32, device=dev)
    out_o = torch.empty(max(kc, 1), dtype=torch.int32, device=dev)
    out_i = torch.empty(max(ic, 1), dtype=torch.int32, device=dev)
    counts = torch.zeros(4, dtype=torch.int32, device=dev)
    wsb = int(lib.wah_append_workspace_bytes(ka, kb))
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    rc = lib.wah_append(ak.data_ptr(), ao.data_ptr(), ai.data_ptr(), ka, la, rows_a,
                        bk.data_ptr(), bo.data_ptr(), bi.data_ptr(), kb, lb, out_k.data_ptr(),
                        out_o.data_ptr(), out_i.data_ptr(), max(kc, 1), max(ic, 1),
                        counts.data_ptr(), ws.data_ptr(), wsb, _stream_handle(stream))
    _check(rc, "wah_append")
    c = counts.cpu().numpy().view(np.uint32)
    if c[3] != WAH_OK:
        raise WahError(int(c[3]), "wah_append (device)")
    K, L = int(c[0]), int(c[1])
    return WahIndex(out_k[:K], out_o[:K], out_i[:L], 0)


def _term(t):
    if t is None:
        return 0, 0
    if isinstance(t, (tuple, list)):
        return int(t[0]), int(t[1])
    return int(t), int(t)


def query(idx: WahIndex, n: int, a, op: int = QUERY_KEYS, b=None, words: bool = True,
          rows: bool = True, stream=None):
    """Rows of ``idx`` (an index of ``n`` rows) whose value lies in term A
    (a value ``v`` or an inclusive range ``(lo, hi)``), combined with term B
    by ``op`` (QUERY_OR / QUERY_AND / QUERY_ANDNOT; QUERY_KEYS = A alone).

    Returns ``(words, rows)``: the result as a WAH bitmap in the index's own
    format and as ascending row ids (CUDA int32 tensors, uint32 bits; None
    for an output not asked for)."""
    lib = _lib.load()
    torch = _torch()
    keys, offsets, index, dev = _index_tensors(idx)
    K, L = len(idx.keys), len(idx.index)
    a_lo, a_hi = _term(a)
    b_lo, b_hi = _term(b)
    nchunks = (n + 30) // 31
    wcap = 2 * nchunks
    w_out = torch.empty(max(wcap, 1), dtype=torch.int32, device=dev) if words else None
    r_out = torch.empty(max(n, 1), dtype=torch.int32, device=dev) if rows else None
    res = torch.zeros(4, dtype=torch.int32, device=dev)
    wsb = int(lib.wah_query_workspace_bytes(n))
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    rc = lib.wah_query(keys.data_ptr(), offsets.data_ptr(), index.data_ptr(), K, L, n, a_lo, a_hi,
                       op, b_lo, b_hi, w_out.data_ptr() if words else None, wcap,
                       r_out.data_ptr() if rows else None, n, res.data_ptr(), ws.data_ptr(), wsb,
                       _stream_handle(stream))
    _check(rc, "wah_query")
    r = res.cpu().numpy().view(np.uint32)
    if r[2] != WAH_OK:
        raise WahError(int(r[2]), "wah_query (device)")
    nw, nr = int(r[0]), int(r[1])
    return (w_out[:nw] if words else None), (r_out[:nr] if rows else None)


def sort_rids_by_value(values, bound: int = 0, stream=None, device="cuda"):
    """Phase a1: (sorted values, rids) as CUDA int32 tensors (uint32 bits)."""
    lib = _lib.load()
    torch = _torch()
    v = _as_device_u32(values, device)
    n = v.numel()
    out_v = torch.empty(max(n, 1), dtype=torch.int32, device=v.device)
    out_r = torch.empty(max(n, 1), dtype=torch.int32, device=v.device)
    status = torch.zeros(4, dtype=torch.int32, device=v.device)
    wsb = workspace_bytes(max(n, 1), bound)
    ws = torch.empty(wsb, dtype=torch.uint8, device=v.device)
    rc = lib.wah_sort_rids_by_value(v.data_ptr(), n, bound, out_v.data_ptr(), out_r.data_ptr(),
                                    status.data_ptr(), ws.data_ptr(), wsb,
                                    _stream_handle(stream))
    _check(rc, "wah_sort_rids_by_value")
    st = int(status[0].item())
    if st != WAH_OK:
        raise WahError(st, "wah_sort_rids_by_value (device)")
    return out_v[:n], out_r[:n]


def build_sorted(sorted_values, rids, stream=None) -> WahIndex:
    """Phases a2..a6 on an already sorted (value, rid) stream."""
    lib = _lib.load()
    torch = _torch()
    sv = _as_device_u32(sorted_values, "cuda")
    sr = _as_device_u32(rids, sv.device)
    n = sv.numel()
    b = _Buffers(n, 0, sv.device)
    rc = lib.wah_build_sorted(sv.data_ptr(), sr.data_ptr(), n, b.keys.data_ptr(),
                              b.offsets.data_ptr(), b.index.data_ptr(), b.counts.data_ptr(),
                              b.ws.data_ptr(), b.ws_bytes, _stream_handle(stream))
    _check(rc, "wah_build_sorted")
    c = b.counts.cpu().numpy().view(np.uint32)
    if c[3] != WAH_OK:
        raise WahError(int(c[3]), "wah_build_sorted (device)")
    K, L, k = int(c[0]), int(c[1]), int(c[2])
    return WahIndex(b.keys[:K], b.offsets[:K], b.index[:L], k)


class HostContext:
    """Host buffers in, host buffers out, through ``wah_ctx_build_host``.

    Device buffers for columns up to ``max_n`` rows are allocated once and
    reused; each :meth:`build` copies the values in, builds, and copies keys,
    offsets and index out (the reference ``phases`` flow,
    src/phases.cpp:720-1088).
    """

    def __init__(self, max_n: int, bound: int = 0):
        self._lib = _lib.load()
        self.max_n = max_n
        self.bound = bound
        h = ctypes.c_void_p()
        _check(self._lib.wah_ctx_create(max_n, bound, ctypes.byref(h)), "wah_ctx_create")
        self._h = h
        self.keys_cap, self.index_cap = output_caps(max(max_n, 1), bound)

    def close(self):
        if self._h:
            self._lib.wah_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def build_into(self, values: np.ndarray, keys: np.ndarray, offsets: np.ndarray,
                   index: np.ndarray) -> wah_counts:
        """Build into caller-provided host arrays (pinned arrays are fastest)."""
        v = np.ascontiguousarray(values, dtype=np.uint32)
        cnt = wah_counts()
        rc = self._lib.wah_ctx_build_host(self._h, v.ctypes.data, v.size, keys.ctypes.data,
                                          offsets.ctypes.data, index.ctypes.data,
                                          ctypes.byref(cnt))
        _check(rc, "wah_ctx_build_host")
        return cnt

    def build(self, values: np.ndarray) -> WahIndex:
        keys = np.empty(self.keys_cap, np.uint32)
        offs = np.empty(self.keys_cap, np.uint32)
        index = np.empty(self.index_cap, np.uint32)
        c = self.build_into(values, keys, offs, index)
        return WahIndex(keys[:c.keycnt], offs[:c.keycnt], index[:c.index_len], c.merged)


class Batch:
    """Many device columns built by one launch sequence (``wah_batch_*``).

    ``Batch(sizes, bounds)`` plans the batch; ``set_columns(values)`` takes a
    list of CUDA int32 tensors with those sizes and allocates their outputs;
    ``build()`` (or ``launch_graph()``, a replayed CUDA graph) enqueues the
    build; ``results()`` returns one :class:`WahIndex` per column.
    """

    def __init__(self, sizes, bounds=None, tuning: int = 0):
        self._lib = _lib.load()
        self.sizes = [int(x) for x in sizes]
        self.bounds = [int(x) for x in (bounds if bounds is not None else [0] * len(self.sizes))]
        nc = len(self.sizes)
        ns = (ctypes.c_uint64 * nc)(*self.sizes)
        bs = (ctypes.c_uint32 * nc)(*self.bounds)
        h = ctypes.c_void_p()
        _check(self._lib.wah_batch_create_tuned(ns, bs, nc, tuning, ctypes.byref(h)),
               "wah_batch_create")
        self._h = h
        self._cols = None
        self._keep = None

    @property
    def device_bytes(self) -> int:
        return int(self._lib.wah_batch_device_bytes(self._h))

    @property
    def ranges(self) -> int:
        return int(self._lib.wah_batch_ranges(self._h))

    def set_columns(self, values, stream=None, outputs=None):
        """values: list of CUDA int32 tensors; outputs: optional list of
        (keys, offsets, index, counts) CUDA int32 tensors to reuse."""
        torch = _torch()
        nc = len(self.sizes)
        if len(values) != nc:
            raise ValueError("one tensor per planned column")
        cols = (_lib.wah_column * nc)()
        outs = []
        for c, v in enumerate(values):
            if v.numel() != self.sizes[c]:
                raise ValueError(f"column {c}: {v.numel()} rows, planned {self.sizes[c]}")
            if outputs is not None:
                keys, offs, index, counts = outputs[c]
            else:
                kc, ic = output_caps(max(self.sizes[c], 1), self.bounds[c])
                keys = torch.empty(kc, dtype=torch.int32, device=v.device)
                offs = torch.empty(kc, dtype=torch.int32, device=v.device)
                index = torch.empty(ic, dtype=torch.int32, device=v.device)
                counts = torch.zeros(4, dtype=torch.int32, device=v.device)
            outs.append((keys, offs, index, counts))
            cols[c].values = v.data_ptr()
            cols[c].n = self.sizes[c]
            cols[c].bound = self.bounds[c]
            cols[c].keys = keys.data_ptr()
            cols[c].offsets = offs.data_ptr()
            cols[c].index = index.data_ptr()
            cols[c].counts = counts.data_ptr()
        _check(self._lib.wah_batch_set_columns(self._h, cols, _stream_handle(stream)),
               "wah_batch_set_columns")
        self._cols = outs
        self._keep = list(values)
        return outs

    def build(self, stream=None):
        _check(self._lib.wah_batch_build(self._h, _stream_handle(stream)), "wah_batch_build")

    def launch_graph(self, stream=None):
        _check(self._lib.wah_batch_launch_graph(self._h, _stream_handle(stream)),
               "wah_batch_launch_graph")

    def results(self):
        torch = _torch()
        torch.cuda.synchronize()
        out = []
        counts = torch.stack([o[3] for o in self._cols]).cpu().numpy().view(np.uint32)
        for c, (keys, offs, index, _) in enumerate(self._cols):
            K, L, k, st = (int(x) for x in counts[c])
            if st != WAH_OK:
                raise WahError(st, f"batched build, column {c}")
            out.append(WahIndex(keys[:K], offs[:K], index[:L], k))
        return out

    def close(self):
        if self._h:
            self._lib.wah_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching index server (``wah_server_*``).

    ``submit(values, bound, delay)`` queues a pinned host column arriving
    ``delay`` seconds from now and returns an id; ``wait(id)`` blocks until it
    is built and returns its :class:`wah_server_result` (device pointers stay
    valid until ``release(id)``); ``result(id)`` also copies the index out as
    a :class:`WahIndex` of CUDA tensors and releases it.
    """

    def __init__(self, budget_bytes: int = 64 << 30, max_batch: int = 1024, streams: int = 3,
                 plain: bool = False, tuning: int = 0):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        _check(self._lib.wah_server_create_tuned(budget_bytes, max_batch, streams, int(plain),
                                                 tuning, ctypes.byref(h)), "wah_server_create")
        self._h = h
        self._keep = {}

    def submit(self, values, bound: int = 0, delay: float = 0.0) -> int:
        if hasattr(values, "data_ptr"):
            ptr, n = values.data_ptr(), values.numel()
        else:
            ptr, n = values.ctypes.data, values.size
        i = ctypes.c_uint64()
        _check(self._lib.wah_server_submit(self._h, ptr, n, bound, delay, ctypes.byref(i)),
               "wah_server_submit")
        self._keep[i.value] = values
        return i.value

    def wait(self, rid: int):
        res = _lib.wah_server_result()
        rc = self._lib.wah_server_wait(self._h, rid, ctypes.byref(res))
        self._keep.pop(rid, None)
        _check(rc, "wah_server_wait")
        return res

    def release(self, rid: int) -> None:
        _check(self._lib.wah_server_release(self._h, rid), "wah_server_release")

    def result(self, rid: int) -> WahIndex:
        """Wait, copy the outputs into fresh CUDA tensors, release."""
        torch = _torch()
        res = self.wait(rid)
        K, L = res.counts.keycnt, res.counts.index_len
        keys = torch.empty(max(K, 1), dtype=torch.int32, device="cuda")
        offs = torch.empty(max(K, 1), dtype=torch.int32, device="cuda")
        index = torch.empty(max(L, 1), dtype=torch.int32, device="cuda")
        _check(self._lib.wah_server_copy_out(self._h, rid, keys.data_ptr(), offs.data_ptr(),
                                             index.data_ptr(), _stream_handle(None)),
               "wah_server_copy_out")
        torch.cuda.current_stream().synchronize()
        self.release(rid)
        return WahIndex(keys[:K], offs[:K], index[:L], res.counts.merged)

    @property
    def arena_used(self) -> int:
        return int(self._lib.wah_server_arena_used(self._h))

    def close(self):
        if self._h:
            self._lib.wah_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pipeline:
    """Several host-buffer builds in flight (``wah_pipe_*``).

    ``submit`` copies a column in, builds it and copies its index out into
    pinned host buffers owned by this object (one set per slot), without
    waiting; ``result(ticket)`` waits for one build and returns numpy views of
    its outputs (valid until the slot is reused ``depth`` submits later).
    """

    def __init__(self, max_n: int, bound: int = 0, depth: int = 3):
        torch = _torch()
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        _check(self._lib.wah_pipe_create(max_n, bound, depth, ctypes.byref(h)),
               "wah_pipe_create")
        self._h = h
        self.depth = depth
        kc, ic = output_caps(max(max_n, 1), bound)
        self._out = []
        for _ in range(depth):
            self._out.append(dict(
                keys=torch.empty(kc, dtype=torch.int32, pin_memory=True),
                offsets=torch.empty(kc, dtype=torch.int32, pin_memory=True),
                index=torch.empty(ic, dtype=torch.int32, pin_memory=True),
                counts=torch.zeros(4, dtype=torch.int32, pin_memory=True)))
        self._slot_of = {}
        self._next = 0

    def submit(self, values) -> int:
        """values: pinned uint32/int32 host tensor or numpy array (kept alive
        by the caller until the result is taken)."""
        if hasattr(values, "data_ptr"):
            ptr, n = values.data_ptr(), values.numel()
        else:
            ptr, n = values.ctypes.data, values.size
        slot = self._next % self.depth  # the pipe fills its slots round robin
        o = self._out[slot]
        t = ctypes.c_uint64()
        _check(self._lib.wah_pipe_submit(self._h, ptr, n, o["keys"].data_ptr(),
                                         o["offsets"].data_ptr(), o["index"].data_ptr(),
                                         o["counts"].data_ptr(), ctypes.byref(t)),
               "wah_pipe_submit")
        self._next += 1
        self._slot_of[t.value] = slot
        return t.value

    def wait(self, ticket: int) -> None:
        _check(self._lib.wah_pipe_wait(self._h, ticket), "wah_pipe_wait")

    def result(self, ticket: int) -> WahIndex:
        self.wait(ticket)
        o = self._out[self._slot_of.pop(ticket)]
        c = o["counts"].numpy().view(np.uint32)
        if c[3] != WAH_OK:
            raise WahError(int(c[3]), "pipeline build (device)")
        K, L = int(c[0]), int(c[1])
        return WahIndex(o["keys"].numpy().view(np.uint32)[:K],
                        o["offsets"].numpy().view(np.uint32)[:K],
                        o["index"].numpy().view(np.uint32)[:L], int(c[2]))

    def close(self):
        if self._h:
            self._lib.wah_pipe_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def decoded_bitmap(words) -> str:
    """One key's words decoded to a '0'/'1' string, trailing zeros trimmed
    (src/cpu.cpp:47-74)."""
    w = np.asarray(words.cpu().numpy() if hasattr(words, "cpu") else words).view(np.uint32)
    parts = []
    for block in w.tolist():
        if block & 0x80000000:
            parts.append("".join("1" if (block >> i) & 1 else "0" for i in range(31)))
        else:
            bit = "1" if block & 0x40000000 else "0"
            parts.append(bit * (31 * (block & 0x3FFFFFFF)))
    return "".join(parts).rstrip("0")
