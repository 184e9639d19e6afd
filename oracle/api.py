"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

``build()`` compiles ``hbx_oracle.cpp`` with g++ into ``oracle/_build`` and,
where the reference checkout exists, the reference's own kernel into
``oracle/_ref`` (``ref/build_ref.sh``).  ``run_block`` is the end-to-end oracle:
partition + brute-force pair evaluation, returning sorted (left row, right row)
pairs.  ``run_ref_block`` drives the reference's own compiled kernel.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "libhbx_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libhb_ref.so")

def _reference_root() -> str:
    """The reference checkout: $HBX_REFERENCE_ROOT, else a ``reference``
    directory beside this repository (where the build container keeps it);
    the GPU machines have neither, and use what was built or committed."""
    env = os.environ.get("HBX_REFERENCE_ROOT")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


REFERENCE_ROOT = _reference_root()

_lib: Optional[ctypes.CDLL] = None
_ref: Optional[ctypes.CDLL] = None


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "hbx_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(
            ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
             src, "-o", LIB_PATH + ".tmp"]
        )
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    if os.path.exists(os.path.join(REFERENCE_ROOT, "core", "gpu", "global_func.cuh")):
        if force or not os.path.exists(REF_LIB_PATH):
            subprocess.check_call(["bash", os.path.join(HERE, "ref", "build_ref.sh"), REFERENCE_ROOT])
    return LIB_PATH


class HboTable(ctypes.Structure):
    _fields_ = [
        ("n_rows", ctypes.c_int64),
        ("n_cols", ctypes.c_int32),
        ("cell_ptr", ctypes.POINTER(ctypes.c_char_p)),
        ("cell_len", ctypes.POINTER(ctypes.c_int64)),
    ]


class HboStats(ctypes.Structure):
    _fields_ = [
        ("pairs_covered", ctypes.c_int64),
        ("pair_comparisons", ctypes.c_int64),
        ("n_matches", ctypes.c_int64),
        ("fma_ambiguous", ctypes.c_int64),
        ("long_string_pairs", ctypes.c_int64),
        ("jw_evals", ctypes.c_int64),
        ("fp64_flips", ctypes.c_int64),
        ("fp64_max_abs_diff", ctypes.c_double),
    ]


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.hbo_jaro.restype = ctypes.c_float
        L.hbo_jaro.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_char_p, ctypes.c_int64]
        L.hbo_jw.restype = ctypes.c_double
        L.hbo_jw.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_char_p, ctypes.c_int64,
                             ctypes.c_int]
        L.hbo_jw_fp64.restype = ctypes.c_double
        L.hbo_jw_fp64.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_char_p, ctypes.c_int64]
        L.hbo_std_hash.restype = ctypes.c_uint64
        L.hbo_std_hash.argtypes = [ctypes.c_char_p, ctypes.c_int64]
        L.hbo_sort_rules.restype = None
        L.hbo_partition.restype = None
        L.hbo_partition.argtypes = [ctypes.POINTER(HboTable), ctypes.POINTER(ctypes.c_int),
                                    ctypes.c_char_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_int32)]
        L.hbo_block.restype = ctypes.c_int64
        L.hbo_block.argtypes = [
            ctypes.POINTER(HboTable), ctypes.POINTER(HboTable), ctypes.POINTER(ctypes.c_int),
            ctypes.c_char_p, ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_uint64,
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
            ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32), ctypes.c_int64,
            ctypes.POINTER(HboStats)]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def ref_lib() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_LIB_PATH)
        R.hbref_block_partition.restype = ctypes.c_int64
        _ref = R
    return _ref


class CTable:
    """Row-major (ptr, len) cells, kept alive by this object.

    ``cols`` is column-major: each column a sequence of bytes, or a
    ``(blob uint8 array, int64 offsets)`` pair (n_rows + 1 offsets), the
    layout of the large synthetic tables; blob columns are addressed in
    place, without a Python object per cell."""

    def __init__(self, cols):
        self.n_cols = len(cols)
        if cols and all(isinstance(c, tuple) for c in cols):
            self._init_blobs(cols)
            return
        self.n_rows = len(cols[0]) if cols else 0
        cells = [cols[c][r] for r in range(self.n_rows) for c in range(self.n_cols)]
        self._keep = cells
        n = len(cells)
        self.ptr = (ctypes.c_char_p * max(n, 1))(*cells)
        self.len = (ctypes.c_int64 * max(n, 1))(*[len(x) for x in cells])
        self.t = HboTable(self.n_rows, self.n_cols,
                          ctypes.cast(self.ptr, ctypes.POINTER(ctypes.c_char_p)),
                          ctypes.cast(self.len, ctypes.POINTER(ctypes.c_int64)))

    def _init_blobs(self, cols):
        blobs = [np.ascontiguousarray(b, dtype=np.uint8) for b, _ in cols]
        offs = [np.ascontiguousarray(o, dtype=np.int64) for _, o in cols]
        blobs = [b if b.size else np.zeros(1, np.uint8) for b in blobs]
        self.n_rows = len(offs[0]) - 1
        ptr = np.empty((self.n_rows, self.n_cols), dtype=np.uint64)
        ln = np.empty((self.n_rows, self.n_cols), dtype=np.int64)
        for c, (b, o) in enumerate(zip(blobs, offs)):
            if len(o) - 1 != self.n_rows:
                raise ValueError("columns differ in length")
            ptr[:, c] = np.uint64(b.ctypes.data) + o[:-1].astype(np.uint64)
            ln[:, c] = np.diff(o)
        self._keep = (blobs, offs)
        self.ptr, self.len = ptr, ln
        self.t = HboTable(self.n_rows, self.n_cols,
                          ctypes.cast(ptr.ctypes.data, ctypes.POINTER(ctypes.c_char_p)),
                          ctypes.cast(ln.ctypes.data, ctypes.POINTER(ctypes.c_int64)))


def _plan_arrays(plan):
    n = plan.length
    pi = (ctypes.c_int * n)(*plan.pred_index)
    pt = ctypes.create_string_buffer(bytes(plan.pred_type), n)
    th = (ctypes.c_float * n)(*plan.pred_threshold)
    return n, pi, pt, th


@dataclass
class OracleResult:
    pairs: np.ndarray  # (n, 2) uint32, sorted
    pairs_covered: int
    pair_comparisons: int
    fma_ambiguous: int
    long_string_pairs: int
    jw_evals: int = 0           # JW evaluations of the run
    fp64_flips: int = 0         # of them, threshold decisions that differ in FP64
    fp64_max_abs_diff: float = 0.0  # max |JW reference path - JW FP64|


def run_block(left: CTable, right: CTable, plan, n_partitions: int,
              prefix_idx: int = 2147483647, fma_mode: int = 1, n_threads: int = 0,
              left_row_filter: Optional[np.ndarray] = None) -> OracleResult:
    L = lib()
    if n_threads <= 0:
        n_threads = os.cpu_count() or 1
    n, pi, pt, th = _plan_arrays(plan)
    cap = 1 << 16
    filt = None
    if left_row_filter is not None:
        filt = np.ascontiguousarray(left_row_filter, dtype=np.uint8)
    while True:
        ol = (ctypes.c_uint32 * cap)()
        orr = (ctypes.c_uint32 * cap)()
        st = HboStats()
        got = L.hbo_block(ctypes.byref(left.t), ctypes.byref(right.t), pi, pt, th, n,
                          n_partitions, prefix_idx, fma_mode, n_threads,
                          None if filt is None else filt.ctypes.data, ol, orr, cap,
                          ctypes.byref(st))
        if got >= 0:
            break
        cap = -got
    a = np.zeros((got, 2), dtype=np.uint32)
    if got:
        a[:, 0] = np.frombuffer(ol, dtype=np.uint32, count=got)
        a[:, 1] = np.frombuffer(orr, dtype=np.uint32, count=got)
    return OracleResult(a, st.pairs_covered, st.pair_comparisons, st.fma_ambiguous,
                        st.long_string_pairs, st.jw_evals, st.fp64_flips, st.fp64_max_abs_diff)


def partition(table: CTable, plan, n_partitions: int, prefix_idx: int = 2147483647) -> np.ndarray:
    L = lib()
    n, pi, pt, th = _plan_arrays(plan)
    out = np.zeros(table.n_rows, dtype=np.int32)
    L.hbo_partition(ctypes.byref(table.t), pi, pt, n, n_partitions, prefix_idx,
                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    return out


def run_ref_block(left: CTable, right: CTable, plan, n_partitions: int,
                  prefix_idx: int = 2147483647, n_threads: int = 0) -> List[Tuple[bytes, bytes]]:
    """The reference's own blocking_kernel, partition by partition.

    Returns sorted (id_l, id_r) byte pairs as the reference writes them.
    """
    R = ref_lib()
    if n_threads <= 0:
        n_threads = os.cpu_count() or 1
    bl = partition(left, plan, n_partitions, prefix_idx)
    br = partition(right, plan, n_partitions, prefix_idx)
    n, pi, pt, th = _plan_arrays(plan)
    out: List[Tuple[bytes, bytes]] = []
    for p in range(n_partitions):
        rl = np.nonzero(bl == p)[0].astype(np.int64)
        rr = np.nonzero(br == p)[0].astype(np.int64)
        if len(rl) == 0 or len(rr) == 0:
            continue
        cap = 1 << 16
        while True:
            buf = ctypes.create_string_buffer(cap * 128)
            got = R.hbref_block_partition(
                ctypes.c_int32(left.n_cols), left.ptr, left.len,
                rl.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), ctypes.c_int64(len(rl)),
                ctypes.c_int32(right.n_cols), right.ptr, right.len,
                rr.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), ctypes.c_int64(len(rr)),
                pi, pt, th, ctypes.c_int(n), ctypes.c_int(n_threads), buf, ctypes.c_int64(cap))
            if got >= 0:
                break
            cap = int(-got) + 16
        raw = buf.raw
        for i in range(got):
            s = raw[i * 128:(i + 1) * 128]
            out.append((s[:64].split(b"\0", 1)[0], s[64:].split(b"\0", 1)[0]))
    out.sort()
    return out
