"""GB300 rule-based blocking engine -- Python binding of ``libhbx.so``.

The engine is a drop-in for HyperBlocker's pair-evaluation path: same CLI
flags, YAML rules, CSV inputs and ``id_l,id_r`` output file, with the pair
evaluation running as hand-written sm_103a CUDA behind the C ABI declared in
``include/hbx.h``.  This module only marshals arguments through ctypes; there
is no Python or CPU fallback, and loading fails loudly when the library has
not been built (``python -m hyperblocker_gb300.build``).

Mirrors of the reference's interfaces:

* :class:`HyperBlocker` -- ``core/hyperblocker.cuh:45-131`` (constructor
  arguments and ``Run()``), writing the output file like
  ``core/components/host_reducer.h:80-90``;
* :func:`run_cli` -- ``examples/run_hyperblocker.cu:22-59``;
* :class:`Plan` -- ``core/components/execution_plan_generator.h``
  (``serialized()`` is its ``SerializedExecutionPlan``);
* :class:`Table` -- ``core/components/data_mngr.h:46-79`` CSV ingest;
* :class:`Session` / :func:`block` -- ``HostProducer::AsyncSubmit`` +
  ``blocking_kernel`` for all partitions (``host_producer.h:109-215``,
  ``global_func.cuh:104-185``).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhbx.so")
EXE_PATH = os.path.join(HERE, "_build", "run_hyperblocker_exec")
INT_MAX = 2147483647

OK, ERR_INVALID_ARG, ERR_CUDA, ERR_OOM, ERR_CAPACITY, ERR_WATCHDOG, ERR_PARSE, ERR_IO, \
    ERR_UNSUPPORTED, ERR_TIMEOUT = range(10)
MODE_PLAIN, MODE_BATCHED = 0, 1
_MODES = {"plain": MODE_PLAIN, "batched": MODE_BATCHED}


class HbxError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"hbx status {status}: {message}")
        self.status = status
        self.message = message


class Opts(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("use_graph", ctypes.c_int32),
                ("tile_right", ctypes.c_int32), ("eval_variant", ctypes.c_int32),
                ("pred_order", ctypes.c_int32), ("ingest", ctypes.c_int32),
                ("watchdog_cycles", ctypes.c_uint64)]


class Columns(ctypes.Structure):
    _fields_ = [("n_rows", ctypes.c_int64), ("n_cols", ctypes.c_int32),
                ("data", ctypes.POINTER(ctypes.c_char_p)),
                ("offsets", ctypes.POINTER(ctypes.POINTER(ctypes.c_int64)))]


class Pairs(ctypes.Structure):
    _fields_ = [("l_row", ctypes.c_void_p), ("r_row", ctypes.c_void_p),
                ("capacity", ctypes.c_uint64), ("n_written", ctypes.c_uint64),
                ("n_required", ctypes.c_uint64)]


class Stats(ctypes.Structure):
    _fields_ = [("pairs_covered", ctypes.c_uint64), ("pair_comparisons", ctypes.c_uint64),
                ("n_matches", ctypes.c_uint64), ("fma_ambiguous", ctypes.c_uint64),
                ("long_string_pairs", ctypes.c_uint64), ("n_tiles", ctypes.c_uint64),
                ("n_partitions_used", ctypes.c_uint32), ("n_launches", ctypes.c_uint32),
                ("ms_last_run", ctypes.c_double), ("ms_join", ctypes.c_double),
                ("ms_eval", ctypes.c_double), ("jw_word_ops", ctypes.c_uint64),
                ("h2d_bytes", ctypes.c_uint64), ("ms_create", ctypes.c_double),
                ("ingest_on_device", ctypes.c_uint32), ("tile_right", ctypes.c_uint32),
                ("eval_variant", ctypes.c_uint32), ("n_windows", ctypes.c_uint32),
                ("pairs_scanned", ctypes.c_uint64), ("scan_steps", ctypes.c_uint64),
                ("scan_word_ops", ctypes.c_uint64), ("scan_words", ctypes.c_uint32),
                ("reserved0", ctypes.c_uint32), ("scan_warp_steps", ctypes.c_uint64),
                ("rest_scans", ctypes.c_uint64)]

    def as_dict(self) -> Dict[str, float]:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServeOpts(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("max_inflight", ctypes.c_int32),
                ("max_batch_rows", ctypes.c_int64), ("budget_bytes", ctypes.c_uint64),
                ("tile_right", ctypes.c_int32), ("eval_variant", ctypes.c_int32)]


class ServeResult(ctypes.Structure):
    _fields_ = [("req_id", ctypes.c_uint64), ("status", ctypes.c_int32), ("plan", ctypes.c_int32),
                ("n_pairs", ctypes.c_uint64), ("l_row", ctypes.POINTER(ctypes.c_uint32)),
                ("r_row", ctypes.POINTER(ctypes.c_uint32)), ("pair_comparisons", ctypes.c_uint64),
                ("ms_queued", ctypes.c_double), ("ms_total", ctypes.c_double),
                ("batch_requests", ctypes.c_uint32), ("batch_id", ctypes.c_uint32)]


class ServeStats(ctypes.Structure):
    _fields_ = [("requests_done", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("rows", ctypes.c_uint64), ("pair_comparisons", ctypes.c_uint64),
                ("n_pairs", ctypes.c_uint64), ("ms_device", ctypes.c_double),
                ("budget_bytes", ctypes.c_uint64), ("peak_bytes", ctypes.c_uint64),
                ("resident_bytes", ctypes.c_uint64)]

    def as_dict(self) -> Dict[str, float]:
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every function include/hbx.h declares: name -> (restype, argtypes).
_VP = ctypes.c_void_p
SIGNATURES = {
    "hbx_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(Opts), ctypes.POINTER(_VP)]),
    "hbx_ctx_destroy": (ctypes.c_int, [_VP]),
    "hbx_last_error": (ctypes.c_char_p, [_VP]),
    "hbx_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "hbx_plan_from_rule_dir": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.POINTER(_VP)]),
    "hbx_plan_from_yaml": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_char_p), ctypes.c_int32,
                                          ctypes.POINTER(_VP)]),
    "hbx_plan_serialized": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_int32),
                                           ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)),
                                           ctypes.POINTER(ctypes.POINTER(ctypes.c_char)),
                                           ctypes.POINTER(ctypes.POINTER(ctypes.c_float))]),
    "hbx_plan_n_rules": (ctypes.c_int32, [_VP]),
    "hbx_plan_destroy": (ctypes.c_int, [_VP]),
    "hbx_table_from_csv": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.c_char, ctypes.POINTER(_VP)]),
    "hbx_table_ingest": (ctypes.c_int, [_VP, ctypes.POINTER(Columns), ctypes.POINTER(_VP)]),
    "hbx_table_n_rows": (ctypes.c_int64, [_VP]),
    "hbx_table_n_cols": (ctypes.c_int32, [_VP]),
    "hbx_table_column": (ctypes.c_int, [_VP, ctypes.c_int32, ctypes.POINTER(_VP), ctypes.POINTER(_VP)]),
    "hbx_table_destroy": (ctypes.c_int, [_VP]),
    "hbx_session_create": (ctypes.c_int, [_VP, _VP, _VP, _VP, ctypes.c_uint64, ctypes.c_int64,
                                          ctypes.POINTER(_VP)]),
    "hbx_session_run": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.POINTER(Pairs), _VP]),
    "hbx_session_stats": (ctypes.c_int, [_VP, ctypes.POINTER(Stats)]),
    "hbx_session_destroy": (ctypes.c_int, [_VP]),
    "hbx_block": (ctypes.c_int, [_VP, _VP, _VP, _VP, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int,
                                 ctypes.POINTER(Pairs), ctypes.POINTER(Stats), _VP]),
    "hbx_write_pairs": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP, ctypes.c_uint64, ctypes.c_char_p]),
    "hbx_write_pairs_device": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP, ctypes.c_uint64,
                                              ctypes.c_char_p]),
    "hbx_run_cli": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]),
    "hbx_block_static": (ctypes.c_int, [ctypes.c_int, _VP, _VP, _VP, ctypes.c_uint64,
                                        ctypes.c_int64, ctypes.POINTER(Pairs), _VP,
                                        ctypes.POINTER(Stats)]),
    "hbx_static_last_error": (ctypes.c_char_p, []),
    "hbx_block_streamed": (ctypes.c_int, [_VP, _VP, _VP, _VP, ctypes.c_uint64, ctypes.c_int64,
                                          ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(Pairs),
                                          ctypes.POINTER(Stats)]),
    "hbx_serve_open": (ctypes.c_int, [_VP, ctypes.POINTER(_VP), ctypes.c_int32, _VP,
                                      ctypes.POINTER(ServeOpts), ctypes.POINTER(_VP)]),
    "hbx_serve_submit": (ctypes.c_int, [_VP, ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(Columns)]),
    "hbx_serve_poll": (ctypes.c_int, [_VP, ctypes.c_int32, ctypes.POINTER(ServeResult)]),
    "hbx_serve_get_stats": (ctypes.c_int, [_VP, ctypes.POINTER(ServeStats)]),
    "hbx_serve_close": (ctypes.c_int, [_VP]),
    "hbx_serve_last_error": (ctypes.c_char_p, [_VP]),
}

_lib: Optional[ctypes.CDLL] = None


def lib() -> ctypes.CDLL:
    """The engine library.  Raises if it has not been built: no fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing; build it with "
                               "`python -m hyperblocker_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status: int, ctx=None) -> None:
    if status != OK:
        msg = lib().hbx_last_error(ctx)
        raise HbxError(status, (msg or b"").decode(errors="replace"))


class Context:
    """A CUDA device + stream for the engine (hbx_ctx)."""

    def __init__(self, device: int = 0, use_graph: bool = True, tile_right: int = 0,
                 watchdog_cycles: int = 0, eval_variant: int = 0, pred_order: int = 0,
                 ingest: int = 0):
        o = Opts(ctypes.sizeof(Opts), 1 if use_graph else 0, tile_right, eval_variant,
                 pred_order, ingest, watchdog_cycles)
        h = _VP()
        _check(lib().hbx_ctx_create(device, ctypes.byref(o), ctypes.byref(h)))
        self.h = h

    def close(self) -> None:
        if self.h:
            lib().hbx_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Plan:
    """Rules in the reference's order plus the engine's evaluation order."""

    def __init__(self, handle, ctx: Optional[Context] = None):
        self.h = handle
        self.ctx = ctx

    @classmethod
    def from_rule_dir(cls, rule_dir: str, ctx: Optional[Context] = None) -> "Plan":
        h = _VP()
        c = ctx.h if ctx else None
        _check(lib().hbx_plan_from_rule_dir(c, rule_dir.encode(), ctypes.byref(h)), c)
        return cls(h, ctx)

    @classmethod
    def from_yaml(cls, docs: Sequence[str], ctx: Optional[Context] = None) -> "Plan":
        arr = (ctypes.c_char_p * max(len(docs), 1))(*[d.encode() for d in docs])
        h = _VP()
        c = ctx.h if ctx else None
        _check(lib().hbx_plan_from_yaml(c, arr, len(docs), ctypes.byref(h)), c)
        return cls(h, ctx)

    def serialized(self) -> Tuple[List[int], bytes, List[float]]:
        n = ctypes.c_int32()
        pi = ctypes.POINTER(ctypes.c_int32)()
        pt = ctypes.POINTER(ctypes.c_char)()
        th = ctypes.POINTER(ctypes.c_float)()
        _check(lib().hbx_plan_serialized(self.h, ctypes.byref(n), ctypes.byref(pi),
                                         ctypes.byref(pt), ctypes.byref(th)))
        k = n.value
        return [pi[i] for i in range(k)], bytes(pt[i][0] for i in range(k)), [th[i] for i in range(k)]

    @property
    def n_rules(self) -> int:
        return lib().hbx_plan_n_rules(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().hbx_plan_destroy(self.h)
            self.h = None


class Table:
    """Host table (rows x columns of byte strings), CSV header line included."""

    def __init__(self, handle):
        self.h = handle

    @classmethod
    def from_csv(cls, path: str, sep: str = ",", ctx: Optional[Context] = None) -> "Table":
        h = _VP()
        c = ctx.h if ctx else None
        _check(lib().hbx_table_from_csv(c, path.encode(), sep.encode()[:1] or b",", ctypes.byref(h)), c)
        return cls(h)

    @classmethod
    def from_columns(cls, cols, ctx: Optional[Context] = None) -> "Table":
        """Column-major cells: each column a sequence of bytes, or a
        (blob uint8 array, int64 offsets) pair; the engine copies them."""
        cs, keep = _columns_struct(cols)
        h = _VP()
        c = ctx.h if ctx else None
        _check(lib().hbx_table_ingest(c, ctypes.byref(cs), ctypes.byref(h)), c)
        return cls(h)

    @property
    def n_rows(self) -> int:
        return lib().hbx_table_n_rows(self.h)

    @property
    def n_cols(self) -> int:
        return lib().hbx_table_n_cols(self.h)

    def column(self, c: int):
        """Column c as parsed: (cell bytes back to back as uint8, int64
        offsets of n_rows + 1), copies."""
        b, o = _VP(), _VP()
        _check(lib().hbx_table_column(self.h, c, ctypes.byref(b), ctypes.byref(o)), None)
        n = self.n_rows
        off = np.ctypeslib.as_array(ctypes.cast(o, ctypes.POINTER(ctypes.c_int64)), (n + 1,)).copy()
        nb = int(off[-1])
        data = (np.ctypeslib.as_array(ctypes.cast(b, ctypes.POINTER(ctypes.c_uint8)), (nb,)).copy()
                if nb else np.zeros(0, np.uint8))
        return data, off

    def __del__(self):
        if getattr(self, "h", None):
            lib().hbx_table_destroy(self.h)
            self.h = None


def _columns_struct(cols):
    """hbx_columns over column-major cells: each column is a sequence of bytes
    or a (blob uint8 array, int64 offsets) pair.  Returns (struct, keepalive)."""
    n_cols = len(cols)
    datas, offs = [], []
    n_rows = None
    for col in cols:
        if isinstance(col, tuple):
            blob = np.ascontiguousarray(col[0], dtype=np.uint8)
            off = np.ascontiguousarray(col[1], dtype=np.int64)
            if blob.size == 0:
                blob = np.zeros(1, dtype=np.uint8)
        else:
            joined = b"".join(col)
            blob = np.frombuffer(joined, dtype=np.uint8) if joined else np.zeros(1, np.uint8)
            off = np.zeros(len(col) + 1, dtype=np.int64)
            if len(col):
                off[1:] = np.cumsum([len(x) for x in col])
        rows = len(off) - 1
        if n_rows is not None and rows != n_rows:
            raise ValueError("columns differ in length")
        n_rows = rows
        datas.append(blob)
        offs.append(off)
    data_arr = (ctypes.c_char_p * max(n_cols, 1))(
        *[ctypes.cast(d.ctypes.data, ctypes.c_char_p) for d in datas])
    off_arr = (ctypes.POINTER(ctypes.c_int64) * max(n_cols, 1))(
        *[o.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)) for o in offs])
    cs = Columns(n_rows or 0, n_cols, ctypes.cast(data_arr, ctypes.POINTER(ctypes.c_char_p)),
                 ctypes.cast(off_arr, ctypes.POINTER(ctypes.POINTER(ctypes.c_int64))))
    return cs, (datas, offs, data_arr, off_arr)


class Server:
    """Resident right table answering requests of left records (hbx_serve_*).

    ``plans[k]`` is request plan k.  ``submit`` copies the records and returns
    at once; ``poll`` returns finished requests as dicts with the request id,
    its (left row, right row) pairs sorted, and its timings.
    """

    def __init__(self, ctx: Context, plans: Sequence["Plan"], right: "Table",
                 max_inflight: int = 0, max_batch_rows: int = 0, budget_bytes: int = 0,
                 tile_right: int = 0, eval_variant: int = 0):
        o = ServeOpts(ctypes.sizeof(ServeOpts), max_inflight, max_batch_rows, budget_bytes,
                      tile_right, eval_variant)
        arr = (_VP * len(plans))(*[p.h for p in plans])
        h = _VP()
        _check(lib().hbx_serve_open(ctx.h, arr, len(plans), right.h, ctypes.byref(o),
                                    ctypes.byref(h)), ctx.h)
        self.h = h
        self.ctx = ctx
        self._keep = (list(plans), right)

    def _err(self, st: int) -> None:
        if st != OK:
            msg = lib().hbx_serve_last_error(self.h)
            raise HbxError(st, (msg or b"").decode(errors="replace"))

    def submit(self, req_id: int, plan: int, cols) -> None:
        cs, keep = _columns_struct(cols)
        self._err(lib().hbx_serve_submit(self.h, req_id, plan, ctypes.byref(cs)))

    def poll(self, timeout_ms: int = -1) -> Optional[dict]:
        r = ServeResult()
        st = lib().hbx_serve_poll(self.h, timeout_ms, ctypes.byref(r))
        if st == ERR_TIMEOUT:
            return None
        self._err(st)
        n = int(r.n_pairs)
        pairs = np.zeros((n, 2), dtype=np.uint32)
        if n:
            pairs[:, 0] = np.ctypeslib.as_array(r.l_row, shape=(n,))
            pairs[:, 1] = np.ctypeslib.as_array(r.r_row, shape=(n,))
        return {"id": int(r.req_id), "status": int(r.status), "plan": int(r.plan), "pairs": pairs,
                "comparisons": int(r.pair_comparisons), "ms_queued": r.ms_queued,
                "ms_total": r.ms_total, "batch_requests": int(r.batch_requests),
                "batch_id": int(r.batch_id)}

    def stats(self) -> ServeStats:
        s = ServeStats()
        self._err(lib().hbx_serve_get_stats(self.h, ctypes.byref(s)))
        return s

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().hbx_serve_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _mode(mode) -> int:
    return _MODES[mode] if isinstance(mode, str) else int(mode)


class Session:
    """Both tables encoded for one plan and resident on the GPU."""

    def __init__(self, ctx: Context, plan: Plan, left: Table, right: Table,
                 n_partitions: int = 1, prefix_idx: int = INT_MAX):
        h = _VP()
        _check(lib().hbx_session_create(ctx.h, plan.h, left.h, right.h, n_partitions, prefix_idx,
                                        ctypes.byref(h)), ctx.h)
        self.h = h
        self.ctx = ctx
        self._keep = (plan, left, right)

    def run_device(self, mode, out_l_ptr: int, out_r_ptr: int, capacity: int,
                   stream_ptr: Optional[int] = None) -> int:
        """Runs on device-resident inputs into device buffers; returns matches."""
        p = Pairs(out_l_ptr, out_r_ptr, capacity, 0, 0)
        st = lib().hbx_session_run(self.h, _mode(mode), ctypes.byref(p), stream_ptr)
        if st == ERR_CAPACITY:
            raise HbxError(st, f"needs capacity {p.n_required}")
        _check(st, self.ctx.h)
        return int(p.n_written)

    def count(self, mode, stream_ptr: Optional[int] = None) -> int:
        """Runs once without an output buffer; returns the number of matches
        (the capacity a run_device call needs)."""
        p = Pairs(None, None, 0, 0, 0)
        st = lib().hbx_session_run(self.h, _mode(mode), ctypes.byref(p), stream_ptr)
        if st not in (OK, ERR_CAPACITY):
            _check(st, self.ctx.h)
        return int(p.n_required)

    def stats(self) -> Stats:
        s = Stats()
        _check(lib().hbx_session_stats(self.h, ctypes.byref(s)))
        return s

    def close(self) -> None:
        if self.h:
            lib().hbx_session_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def block(ctx: Context, plan: Plan, left: Table, right: Table, n_partitions: int = 1,
          prefix_idx: int = INT_MAX, mode="batched", capacity: Optional[int] = None,
          stream_ptr: Optional[int] = None, out=None, stack: bool = True):
    """Host tables -> (pairs (n, 2) uint32 of (left row, right row), stats).

    ``hbx_block`` writes nothing when the output buffer is too small (it
    reports the size needed and the call is repeated), so without an explicit
    ``capacity`` the buffer is sized from the largest result seen on this
    context, with a quarter of headroom.  ``out`` = (left rows, right rows),
    two uint32 host arrays the caller keeps between calls, is used when it is
    large enough.  With ``stack=False`` the pairs come back as the two row
    arrays the C ABI fills, (left rows, right rows), views of ``out`` when it
    is given, without the copy into one (n, 2) array.
    """
    if capacity is None:
        capacity = getattr(ctx, "_capacity_hint", 1 << 16)
    while True:
        if out is not None and len(out[0]) >= capacity and len(out[1]) >= capacity:
            ol, orr = out
            capacity = min(len(ol), len(orr))
        else:
            ol = np.empty(max(capacity, 1), dtype=np.uint32)
            orr = np.empty(max(capacity, 1), dtype=np.uint32)
        p = Pairs(ol.ctypes.data, orr.ctypes.data, capacity, 0, 0)
        s = Stats()
        st = lib().hbx_block(ctx.h, plan.h, left.h, right.h, n_partitions, prefix_idx, _mode(mode),
                             ctypes.byref(p), ctypes.byref(s), stream_ptr)
        if st == ERR_CAPACITY:
            capacity = int(p.n_required)
            ctx._capacity_hint = max(getattr(ctx, "_capacity_hint", 0), capacity + capacity // 4)
            continue
        _check(st, ctx.h)
        n = int(p.n_written)
        if n + n // 4 > getattr(ctx, "_capacity_hint", 1 << 16):
            ctx._capacity_hint = n + n // 4
        if not stack:
            return (ol[:n], orr[:n]), s
        return np.stack([ol[:n], orr[:n]], axis=1), s


def block_streamed(ctx: Context, plan: Plan, left: Table, right: Table, n_partitions: int,
                   window_bytes: int, prefix_idx: int = INT_MAX, mode="batched",
                   capacity: Optional[int] = None):
    """``hbx_block_streamed``: partition windows of at most ``window_bytes``
    of device memory, two in flight; returns (pairs (n, 2) uint32, stats)."""
    if capacity is None:
        capacity = getattr(ctx, "_capacity_hint", 1 << 16)
    while True:
        ol = np.empty(max(capacity, 1), dtype=np.uint32)
        orr = np.empty(max(capacity, 1), dtype=np.uint32)
        p = Pairs(ol.ctypes.data, orr.ctypes.data, capacity, 0, 0)
        s = Stats()
        st = lib().hbx_block_streamed(ctx.h, plan.h, left.h, right.h, n_partitions, prefix_idx,
                                      _mode(mode), window_bytes, ctypes.byref(p), ctypes.byref(s))
        if st == ERR_CAPACITY:
            capacity = int(p.n_required)
            ctx._capacity_hint = max(getattr(ctx, "_capacity_hint", 0), capacity + capacity // 4)
            continue
        _check(st, ctx.h)
        n = int(p.n_written)
        return np.stack([ol[:n], orr[:n]], axis=1), s


def write_pairs(left: Table, right: Table, pairs: np.ndarray, path: str,
                ctx: Optional[Context] = None) -> None:
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32)
    l = np.ascontiguousarray(pairs[:, 0]) if len(pairs) else np.zeros(1, np.uint32)
    r = np.ascontiguousarray(pairs[:, 1]) if len(pairs) else np.zeros(1, np.uint32)
    c = ctx.h if ctx else None
    _check(lib().hbx_write_pairs(c, left.h, right.h, l.ctypes.data, r.ctypes.data, len(pairs),
                                 path.encode()), c)


def write_pairs_device(ctx: Context, left: Table, right: Table, l_row_ptr: int, r_row_ptr: int,
                       n: int, path: str) -> None:
    """Appends the id lines of n pairs held in DEVICE memory (two uint32
    arrays given by address), formatted on the device."""
    _check(lib().hbx_write_pairs_device(ctx.h, left.h, right.h, l_row_ptr, r_row_ptr, n,
                                        path.encode()), ctx.h)


def run_cli(argv: Sequence[str]) -> int:
    """``run_hyperblocker_exec`` in-process; argv[0] is the program name."""
    arr = (ctypes.c_char_p * len(argv))(*[a.encode() for a in argv])
    return lib().hbx_run_cli(len(argv), arr)


class HyperBlocker:
    """Mirror of ``sics::hyperblocker::core::HyperBlocker`` (core/hyperblocker.cuh:45-131)."""

    def __init__(self, rule_dir: str, data_path_l: str, data_path_r: str, output_path: str,
                 n_partitions: int, prefix_hash_predicate_index: int = INT_MAX, sep: str = ",",
                 scheduler_type: str = "CHBL", mode: str = "batched", device: int = 0):
        self.ctx = Context(device)
        self.plan = Plan.from_rule_dir(rule_dir, self.ctx)
        self.left = Table.from_csv(data_path_l, sep, self.ctx)
        self.right = Table.from_csv(data_path_r, sep, self.ctx)
        self.output_path = output_path
        self.n_partitions = n_partitions
        self.prefix = prefix_hash_predicate_index
        self.mode = mode
        self.last_stats: Optional[Stats] = None

    def Run(self) -> np.ndarray:
        pairs, st = block(self.ctx, self.plan, self.left, self.right, self.n_partitions,
                          self.prefix, self.mode)
        order = np.lexsort((pairs[:, 1], pairs[:, 0])) if len(pairs) else np.zeros(0, np.int64)
        pairs = pairs[order]
        if self.output_path:
            write_pairs(self.left, self.right, pairs, self.output_path, self.ctx)
        self.last_stats = st
        return pairs
