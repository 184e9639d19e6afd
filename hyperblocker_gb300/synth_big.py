"""Vectorised synthetic tables for the large workloads (1M-20M rows).

Same schema and value distributions as :mod:`hyperblocker_gb300.synth`
(titles of Zipf(1.1) pseudo-words, 20-120 characters; 1-6 "First Last"
authors; categorical venues; years), but every column is produced directly
as one byte blob plus int64 cell offsets -- the layout ``hbx_table_ingest``
takes -- with numpy gathers instead of per-row Python strings, so ten
million rows take seconds rather than minutes.  Tables carry the header row
first, like the CSV files the reference reads.

Workloads:

* :func:`c3`  1M x 1M, 8 rules mixing 1-2 equalities with 1-3 Jaro-Winkler
  predicates (thresholds U[0.80, 0.95]), 64 partitions.  The partition key is
  an extra column ``key`` drawn Zipf(1.3) over 256 values; every two-equality
  rule starts with it, so the reference's rule sort puts it in plan slot 0
  and the hash partitions get heavily uneven sizes.
* :func:`c4_right` / :func:`c4_requests`  the serving workload: a resident
  right table and a seeded trace of left-record requests (log-uniform 1-50k
  rows, Poisson arrivals, one of 4 rules each).

Everything is drawn from PCG64 with base seed 0x48594250 + config number
(only ``integers`` and ``random``).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

from hyperblocker_gb300 import synth

BASE_SEED = synth.BASE_SEED
CHUNK = 1 << 20


@dataclass
class Tokens:
    """A small vocabulary of byte strings as one blob + offsets."""
    blob: np.ndarray  # uint8
    off: np.ndarray   # int64, len + 1
    _pad: Optional[np.ndarray] = None  # zero-padded matrix form, built on first use

    @classmethod
    def of(cls, items: Sequence[bytes]) -> "Tokens":
        off = np.zeros(len(items) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(x) for x in items])
        return cls(np.frombuffer(b"".join(items), dtype=np.uint8).copy(), off)

    @property
    def lens(self) -> np.ndarray:
        return np.diff(self.off)


def _padded(tok: Tokens) -> np.ndarray:
    """Tokens as rows of a zero-padded (n_tokens, width) byte matrix."""
    lens = tok.lens
    width = int(lens.max()) if len(lens) else 1
    mat = np.zeros((len(lens), width), dtype=np.uint8)
    for i in range(len(lens)):
        mat[i, :lens[i]] = tok.blob[tok.off[i]:tok.off[i + 1]]
    return mat


def _join(tok: Tokens, ids: np.ndarray, counts: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Rows made of token sequences: row i = tokens ids[s_i : s_i + counts[i]]
    concatenated.  Returns (blob, offsets)."""
    tl = tok.lens[ids]
    lens = tok.lens
    if len(lens) and lens.max() <= 48 and len(ids) > 4096:
        # gather fixed-width padded rows, then drop the padding: no per-byte
        # index arrays
        if getattr(tok, "_pad", None) is None:
            tok._pad = _padded(tok)
        mat = tok._pad[ids]
        keep = np.arange(mat.shape[1], dtype=np.int64)[None, :] < tl[:, None]
        blob = mat[keep]
        row_end = np.cumsum(counts)
        off = np.zeros(len(counts) + 1, dtype=np.int64)
        ends = np.concatenate([[0], np.cumsum(tl)])
        off[1:] = ends[row_end]
        return blob, off
    total = int(tl.sum())
    starts = np.zeros(len(ids), dtype=np.int64)
    if len(ids) > 1:
        np.cumsum(tl[:-1], out=starts[1:])
    rep = np.repeat(np.arange(len(ids), dtype=np.int64), tl)
    within = np.arange(total, dtype=np.int64) - starts[rep]
    blob = tok.blob[tok.off[ids][rep] + within]
    row_end = np.cumsum(counts)
    off = np.zeros(len(counts) + 1, dtype=np.int64)
    ends = np.concatenate([[0], np.cumsum(tl)])
    off[1:] = ends[row_end]
    return blob, off


class Gen:
    """Column generators sharing one vocabulary and random stream."""

    def __init__(self, config: int):
        self.rng = np.random.Generator(np.random.PCG64(BASE_SEED + config))
        vocab = synth.make_vocab(self.rng)
        self.words = Tokens.of([w.encode() for w in vocab.words])
        self.word_sp = _padded(Tokens.of([w.encode() + b" " for w in vocab.words]))
        first = Tokens.of([f.encode() + b" " for f in vocab.first])
        last = Tokens.of([l.encode() + b", " for l in vocab.last])
        self.first_sp, self.first_sp_len = _padded(first), first.lens
        self.last_cm, self.last_cm_len = _padded(last), last.lens
        self.n_first = len(vocab.first)
        self.n_last = len(vocab.last)
        w = 1.0 / np.arange(1, len(vocab.words) + 1, dtype=np.float64) ** 1.1
        cdf = np.cumsum(w) / w.sum()
        # inverse CDF tabulated on 2^22 equal bins: a draw is one table lookup
        # (the rarest word has probability 2.3e-6, about ten bins)
        u = (np.arange(1 << 22, dtype=np.float64) + 0.5) / (1 << 22)
        self.word_lut = np.minimum(np.searchsorted(cdf, u, side="right"),
                                   len(cdf) - 1).astype(np.int32)

    def _zipf_words(self, k: int) -> np.ndarray:
        return self.word_lut[self.rng.integers(0, 1 << 22, size=k)]

    def titles(self, n: int, lo: int = 20, hi: int = 120) -> Tuple[np.ndarray, np.ndarray]:
        K = 24 if hi <= 120 else 64
        target = self.rng.integers(lo, hi + 1, size=n)
        ids = self._zipf_words(n * K).reshape(n, K)
        wl = self.words.lens[ids]
        cum = np.cumsum(wl + 1, axis=1) - 1  # length when words 0..j are taken
        # words until the target is reached, never past 120 characters
        take = np.ones_like(cum, dtype=bool)
        take[:, 1:] = (cum[:, :-1] < target[:, None]) & (cum[:, 1:] <= hi)
        take = np.logical_and.accumulate(take, axis=1)
        counts = take.sum(axis=1)
        sel = ids[take]
        # each word with its trailing space, except the row's last word
        tl = self.words.lens[sel] + 1
        tl[np.cumsum(counts) - 1] -= 1
        return _rows_from_padded(self.word_sp[sel], tl, counts)

    def authors(self, n: int, kmin: int = 1, kmax: int = 6) -> Tuple[np.ndarray, np.ndarray]:
        k = self.rng.integers(kmin, kmax + 1, size=n)
        m = int(k.sum())
        f = self.rng.integers(0, self.n_first, size=m)
        l = self.rng.integers(0, self.n_last, size=m)
        # "First " + "Last, " per name; the row's last name drops the ", "
        tl = np.empty(2 * m, dtype=np.int64)
        tl[0::2] = self.first_sp_len[f]
        tl[1::2] = self.last_cm_len[l]
        tl[2 * (np.cumsum(k) - 1) + 1] -= 2
        w = max(self.first_sp.shape[1], self.last_cm.shape[1])
        mat = np.zeros((2 * m, w), dtype=np.uint8)
        mat[0::2, :self.first_sp.shape[1]] = self.first_sp[f]
        mat[1::2, :self.last_cm.shape[1]] = self.last_cm[l]
        return _rows_from_padded(mat, tl, 2 * k)


def _rows_from_padded(mat: np.ndarray, tl: np.ndarray, counts: np.ndarray
                      ) -> Tuple[np.ndarray, np.ndarray]:
    """Rows made of consecutive tokens: token t is mat[t, :tl[t]]; row i has
    counts[i] tokens.  Returns (blob, offsets)."""
    keep = np.arange(mat.shape[1], dtype=np.int64)[None, :] < tl[:, None]
    blob = mat[keep]
    ends = np.concatenate([[0], np.cumsum(tl)])
    off = np.zeros(len(counts) + 1, dtype=np.int64)
    off[1:] = ends[np.cumsum(counts)]
    return blob, off


def _categorical(values: Sequence[bytes], idx: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    tok = Tokens.of(values)
    return _join(tok, idx.astype(np.int64), np.ones(len(idx), dtype=np.int64))


def _ids(base: int, n: int) -> Tuple[np.ndarray, np.ndarray]:
    v = base + np.arange(n, dtype=np.int64)
    digits = np.stack([(v // 10 ** k) % 10 for k in range(8, -1, -1)], axis=1).astype(np.uint8) + 48
    return digits.reshape(-1), np.arange(n + 1, dtype=np.int64) * 9


def _concat(parts: List[Tuple[np.ndarray, np.ndarray]]) -> Tuple[np.ndarray, np.ndarray]:
    blobs, offs, base = [], [np.zeros(1, dtype=np.int64)], 0
    for b, o in parts:
        blobs.append(b)
        offs.append(o[1:] + base)
        base += int(o[-1])
    return (np.concatenate(blobs) if blobs else np.zeros(0, np.uint8)), np.concatenate(offs)


@dataclass
class BlobTable:
    """Column blobs + offsets, header row first (what hbx_table_ingest takes)."""
    names: List[str]
    cols: List[Tuple[np.ndarray, np.ndarray]]

    @property
    def n_rows(self) -> int:
        return len(self.cols[0][1]) - 1

    def cell(self, c: int, r: int) -> bytes:
        b, o = self.cols[c]
        return b[o[r]:o[r + 1]].tobytes()

    def rows(self, idx: Sequence[int]) -> List[List[bytes]]:
        """Column-major cells of the given rows (for the oracle on samples)."""
        return [[self.cell(c, int(r)) for r in idx] for c in range(len(self.cols))]

    def to_columns(self) -> List[List[bytes]]:
        return self.rows(range(self.n_rows))


def _with_header(names: Sequence[str], cols: List[Tuple[np.ndarray, np.ndarray]]) -> BlobTable:
    out = []
    for name, (b, o) in zip(names, cols):
        h = name.encode()
        out.append((np.concatenate([np.frombuffer(h, np.uint8), b]),
                    np.concatenate([[0], o + len(h)]).astype(np.int64)))
    return BlobTable(list(names), out)


VENUES = [v.encode() for v in synth._venue_names(BASE_SEED + 102, 500)]
YEARS = [str(y).encode() for y in range(1980, 2006)]


def _venue_idx(rng, n: int) -> np.ndarray:
    w = 1.0 / np.arange(1, 501) ** 1.0
    cdf = np.cumsum(w) / w.sum()
    return np.minimum(np.searchsorted(cdf, rng.random(n), side="right"), 499)


def _key_idx(rng, n: int, n_keys: int = 256, s: float = 1.3) -> np.ndarray:
    w = 1.0 / np.arange(1, n_keys + 1) ** s
    cdf = np.cumsum(w) / w.sum()
    return np.minimum(np.searchsorted(cdf, rng.random(n), side="right"), n_keys - 1)


KEYS = [f"k{i:03d}".encode() for i in range(256)]


def make_rows(g: Gen, n: int, id_base: int, with_key: bool) -> List[Tuple[np.ndarray, np.ndarray]]:
    """n data rows: id, title, authors, venue, year (, key), in chunks."""
    parts: List[List[Tuple[np.ndarray, np.ndarray]]] = [[] for _ in range(6 if with_key else 5)]
    for s in range(0, n, CHUNK):
        k = min(CHUNK, n - s)
        parts[0].append(_ids(id_base + s, k))
        parts[1].append(g.titles(k))
        parts[2].append(g.authors(k))
        parts[3].append(_categorical(VENUES, _venue_idx(g.rng, k)))
        parts[4].append(_categorical(YEARS, g.rng.integers(0, len(YEARS), size=k)))
        if with_key:
            parts[5].append(_categorical(KEYS, _key_idx(g.rng, k)))
    return [_concat(p) for p in parts]


def perturbed_copies(g: Gen, src: BlobTable, rows: np.ndarray, id_base: int
                     ) -> List[Tuple[np.ndarray, np.ndarray]]:
    """Copies of src's data rows (header excluded: row r is table row r + 1)
    with 5% character edits and title token swaps, as synth.make_tables."""
    n = len(rows)
    cols: List[List[bytes]] = [[] for _ in range(len(src.cols))]
    for r in rows:
        r = int(r) + 1
        cols[1].append(synth._swap_tokens(g.rng, synth._edit(g.rng, src.cell(1, r).decode())).encode())
        cols[2].append(synth._edit(g.rng, src.cell(2, r).decode()).encode())
        for c in range(3, len(src.cols)):
            cols[c].append(src.cell(c, r))
    out = [_ids(id_base, n)]
    for c in range(1, len(src.cols)):
        out.append(_join(Tokens.of(cols[c]), np.arange(n, dtype=np.int64), np.ones(n, np.int64)))
    return out


def _append(a: List[Tuple[np.ndarray, np.ndarray]], b: List[Tuple[np.ndarray, np.ndarray]]):
    return [_concat([x, y]) for x, y in zip(a, b)]


NAMES5 = ["id", "title", "authors", "venue", "year"]
NAMES6 = NAMES5 + ["key"]


@dataclass
class BigWorkload:
    name: str
    left: BlobTable
    right: BlobTable
    rules: List[str]
    n_partitions: int
    description: str = ""


def c3(n_left: int = 1_000_000, n_right: int = 1_000_000, n_true: int = 20_000) -> BigWorkload:
    """1M x 1M rows (sizes adjustable for tests), 8 rules, 64 partitions."""
    g = Gen(3)
    left = _with_header(NAMES6, make_rows(g, n_left, 10_000_000, True))
    n_true = min(n_true, n_left, n_right)
    src = np.sort(g.rng.integers(0, n_left, size=n_true))
    right_rows = make_rows(g, n_right - n_true, 50_000_000, True)
    right = _with_header(NAMES6, _append(right_rows, perturbed_copies(
        g, left, src, 50_000_000 + n_right - n_true)))
    thr = np.round(0.80 + 0.15 * g.rng.random(14), 2)
    T, A, V, Y, K = 1, 2, 3, 4, 5
    sims = [[(T, thr[0])], [(A, thr[1]), (T, thr[2])], [(T, thr[3]), (A, thr[4]), (V, thr[5])],
            [(T, thr[6])], [(T, thr[7]), (A, thr[8])], [(T, thr[9])], [(A, thr[10]), (T, thr[11])],
            [(A, thr[12]), (T, thr[13])]]
    eqs = [[K, Y], [K, V], [K, Y], [K, V], [Y], [V], [Y], [V]]
    rules = [rule_yaml6(e, s) for e, s in zip(eqs, sims)]
    return BigWorkload("c3_1Mx1M_8rules_64parts", left, right, rules, 64,
                       "8 rules (4 with key+year/venue equalities, 4 with year or venue), "
                       "1-3 JW predicates, thresholds U[0.80,0.95], key ~ Zipf(1.3) over 256")


def rule_yaml6(eq_cols: Sequence[int], sims: Sequence[tuple]) -> str:
    """synth.rule_yaml for the 6-column schema (id, title, authors, venue, year, key)."""
    doc = synth.rule_yaml(eq_cols, [(c, float(t)) for c, t in sims])
    return doc.replace("[0, 0, 1, 2, 3, 4]", "[0, 0, 1, 2, 3, 4, 5]").replace(
        "[1, 0, 1, 2, 3, 4]", "[1, 0, 1, 2, 3, 4, 5]")


# ------------------------------------------------------- long strings (C5)
def _zipf_key_idx(rng, n: int, n_keys: int, s: float = 1.0) -> np.ndarray:
    w = 1.0 / np.arange(1, n_keys + 1, dtype=np.float64) ** s
    cdf = np.cumsum(w) / w.sum()
    return np.minimum(np.searchsorted(cdf, rng.random(n), side="right"), n_keys - 1)


def _c5_rows(g: Gen, n: int, id_base: int, key_perm: np.ndarray) -> List[Tuple[np.ndarray, np.ndarray]]:
    parts: List[List[Tuple[np.ndarray, np.ndarray]]] = [[] for _ in range(4)]
    for s0 in range(0, n, CHUNK):
        k = min(CHUNK, n - s0)
        parts[0].append(_ids(id_base + s0, k))
        parts[1].append(g.titles(k, 64, 256))
        parts[2].append(g.authors(k, 5, 16))
        # the blocking key: a uint32 per bucket, written as decimal text
        keys = key_perm[_zipf_key_idx(g.rng, k, len(key_perm))]
        parts[3].append(_join(Tokens.of([b"%d" % x for x in np.unique(keys)]),
                              np.searchsorted(np.unique(keys), keys).astype(np.int64),
                              np.ones(k, dtype=np.int64)))
    return [_concat(p) for p in parts]


NAMES_C5 = ["id", "title", "authors", "key"]


def c5(n_left: int = 1_000_000, n_right: int = 1_000_000, n_true: int = 20_000,
       n_keys: int = 1 << 20) -> BigWorkload:
    """Long strings: titles 64-256 and authors of 5-16 names (about 64-256
    characters), an equality key of n_keys uint32 values with Zipf(1.0)
    occupancy, 3 rules, 64 partitions.  The quoted configuration is 20M x 20M;
    sizes are parameters."""
    g = Gen(5)
    key_perm = g.rng.integers(0, 1 << 32, size=n_keys, dtype=np.uint64)
    left = _with_header(NAMES_C5, _c5_rows(g, n_left, 20_000_000, key_perm))
    n_true = min(n_true, n_left, n_right)
    src = np.sort(g.rng.integers(0, n_left, size=n_true))
    right_rows = _c5_rows(g, n_right - n_true, 60_000_000, key_perm)
    right = _with_header(NAMES_C5, _append(right_rows, perturbed_copies(
        g, left, src, 60_000_000 + n_right - n_true)))
    T, A, K = 1, 2, 3
    rules = [rule_yaml_c5([K], [(T, 0.95)]), rule_yaml_c5([K], [(A, 0.94)]),
             rule_yaml_c5([K], [(T, 0.92), (A, 0.92)])]
    return BigWorkload("c5_long_strings", left, right, rules, 64,
                       "3 rules on a Zipf(1.0) key over 2^20 values: JW(title)>=0.95 | "
                       "JW(authors)>=0.94 | JW(title)>=0.92 and JW(authors)>=0.92")


def rule_yaml_c5(eq_cols: Sequence[int], sims: Sequence[tuple]) -> str:
    """synth.rule_yaml for the 4-column schema (id, title, authors, key)."""
    doc = synth.rule_yaml(eq_cols, [(c, float(t)) for c, t in sims])
    return doc.replace("[0, 0, 1, 2, 3, 4]", "[0, 0, 1, 2, 3]").replace(
        "[1, 0, 1, 2, 3, 4]", "[1, 0, 1, 2, 3]")


# ---------------------------------------------------------------- serving (C4)
SERVE_RULES = [
    synth.rule_yaml([4, 3], [(1, 0.89)]),
    synth.rule_yaml([4, 3], [(2, 0.85), (1, 0.8)]),
    synth.rule_yaml([3, 4], [(1, 0.95)]),
    synth.rule_yaml([4, 3], [(1, 0.85), (2, 0.9)]),
]


def c4_right(n_right: int = 10_000_000) -> BlobTable:
    g = Gen(4)
    return _with_header(NAMES5, make_rows(g, n_right, 100_000_000, False))


@dataclass
class Request:
    t_arrival: float  # seconds from the start of the trace
    rule: int
    cols: List[Tuple[np.ndarray, np.ndarray]]  # column blobs + offsets, no header row

    @property
    def n_rows(self) -> int:
        return len(self.cols[0][1]) - 1


def c4_requests(right: BlobTable, n_requests: int, rate: float = 200.0, min_rows: int = 1,
                max_rows: int = 50_000, seed: int = 0, p_true: float = 0.02,
                sizes: Optional[Sequence[int]] = None) -> List[Request]:
    """Poisson arrivals; sizes log-uniform in [min_rows, max_rows] (or given);
    each request is a fresh set of left records of which a fraction p_true are
    perturbed copies of right rows (so that matches exist), appended last."""
    g = Gen(40 + seed)
    gaps = -np.log(1.0 - g.rng.random(n_requests)) / rate
    t = np.cumsum(gaps)
    if sizes is None:
        lo, hi = np.log(min_rows), np.log(max_rows + 1)
        sz = np.exp(lo + (hi - lo) * g.rng.random(n_requests)).astype(np.int64)
        sizes = np.clip(sz, min_rows, max_rows)
    rules = g.rng.integers(0, len(SERVE_RULES), size=n_requests)
    out = []
    for i in range(n_requests):
        n = int(sizes[i])
        k = min(n, int(round(n * p_true)))
        base = 900_000_000 + 100_000 * i
        cols = make_rows(g, n - k, base, False)
        if k:
            src = g.rng.integers(0, right.n_rows - 1, size=k)
            cols = _append(cols, perturbed_copies(g, right, src, base + n - k))
        out.append(Request(float(t[i]), int(rules[i]), cols))
    return out


def write_files(w: BigWorkload, out_dir: str) -> None:
    """Writes a workload as the reference's CLI reads it: l.csv and r.csv
    (every cell quoted, the header line first) and rules/<k>.yaml."""
    import os

    os.makedirs(os.path.join(out_dir, "rules"), exist_ok=True)
    for name, t in (("l.csv", w.left), ("r.csv", w.right)):
        with open(os.path.join(out_dir, name), "wb") as f:
            for i in range(t.n_rows):  # the header line is row 0
                f.write(b",".join(b'"' + bytes(b[o[i]:o[i + 1]]) + b'"' for b, o in t.cols) + b"\n")
    for k, doc in enumerate(w.rules):
        with open(os.path.join(out_dir, "rules", f"{k}.yaml"), "w") as f:
            f.write(doc)


if __name__ == "__main__":
    # python -m hyperblocker_gb300.synth_big c3|c5 ROWS OUT_DIR: the workload at
    # ROWS x ROWS as CSV files and a rule directory; prints its partition count
    import sys

    kind, n, out = sys.argv[1], int(sys.argv[2]), sys.argv[3]
    wl = (c3 if kind == "c3" else c5)(n, n, max(1, n // 50))
    write_files(wl, out)
    print(wl.n_partitions)
