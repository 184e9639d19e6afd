"""Seeded synthetic bibliographic tables and rule sets for the blocking engine.

The reference's own data (public DBLP-ACM / DBLP-Google tables) is not
redistributed here; these generators produce tables with the same schema and
the shapes the workloads are quoted on:

* schema ``id`` (int), ``title`` (ASCII words, Zipf(1.1) over a 20k-word
  vocabulary of pseudo-words, 20-120 chars), ``authors`` (1-6 "First Last"
  names joined by ", "), ``venue`` (categorical), ``year`` (int);
* true pairs copy a left row into the right table with per-character edits
  at 5% (substitute / insert / delete, equiprobable) and a swap of two
  adjacent title words with probability 0.1;
* CSVs are written with a header line (the reference reads it as a data row)
  and every string field quoted, like the DBLP-ACM files.

Everything is drawn from numpy's PCG64 with base seed 0x48594250 + config
number, so every machine regenerates identical bytes.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

BASE_SEED = 0x48594250
LETTERS = np.frombuffer(b"abcdefghijklmnopqrstuvwxyz", dtype=np.uint8)


def _pseudo_words(rng: np.random.Generator, n: int, lo: int, hi: int, cap: bool = False) -> List[str]:
    lens = rng.integers(lo, hi + 1, size=n)
    pool = rng.integers(0, 26, size=int(lens.sum()))
    out, pos = [], 0
    for L in lens:
        w = LETTERS[pool[pos:pos + L]].tobytes().decode()
        pos += L
        out.append(w.capitalize() if cap else w)
    return out


def _zipf_sampler(rng: np.random.Generator, n_values: int, s: float):
    w = 1.0 / np.arange(1, n_values + 1, dtype=np.float64) ** s
    cdf = np.cumsum(w)
    cdf /= cdf[-1]

    def draw(k: int) -> np.ndarray:
        return np.minimum(np.searchsorted(cdf, rng.random(k), side="right"), n_values - 1)

    return draw


@dataclass
class Vocab:
    words: List[str]
    first: List[str]
    last: List[str]


def make_vocab(rng: np.random.Generator) -> Vocab:
    words = _pseudo_words(rng, 20000, 2, 10)
    first = _pseudo_words(rng, 600, 3, 8, cap=True)
    last = _pseudo_words(rng, 3000, 4, 10, cap=True)
    return Vocab(words, first, last)


def _titles(rng, vocab: Vocab, n: int) -> List[str]:
    target = rng.integers(20, 121, size=n)
    draw = _zipf_sampler(rng, len(vocab.words), 1.1)
    idx = draw(n * 24)
    out, pos = [], 0
    W = vocab.words
    for t in target:
        parts, L = [], 0
        while True:
            if pos >= len(idx):
                idx = draw(n * 8)
                pos = 0
            w = W[idx[pos]]
            pos += 1
            add = len(w) + (1 if parts else 0)
            if parts and L + add > t:
                break
            parts.append(w)
            L += add
            if L >= t:
                break
        s = " ".join(parts)
        if len(s) < 20:
            s = (s + " " + W[idx[pos % len(idx)]] * 3)[:max(20, len(s))]
        out.append(s[:120].rstrip() or "x" * 20)
    return out


def _authors(rng, vocab: Vocab, n: int) -> List[str]:
    k = rng.integers(1, 7, size=n)
    f = rng.integers(0, len(vocab.first), size=int(k.sum()))
    l = rng.integers(0, len(vocab.last), size=int(k.sum()))
    out, pos = [], 0
    for c in k:
        out.append(", ".join(f"{vocab.first[f[pos + j]]} {vocab.last[l[pos + j]]}" for j in range(c)))
        pos += c
    return out


def _edit(rng, s: str, p: float = 0.05) -> str:
    if not s:
        return s
    b = bytearray(s.encode())
    u = rng.random(len(b))
    ops = rng.integers(0, 3, size=len(b))
    ch = rng.integers(0, 26, size=len(b))
    out = bytearray()
    for i, c in enumerate(b):
        if u[i] >= p:
            out.append(c)
        elif ops[i] == 0:  # substitute
            out.append(int(LETTERS[ch[i]]))
        elif ops[i] == 1:  # insert before
            out.append(int(LETTERS[ch[i]]))
            out.append(c)
        # ops 2: delete
    return out.decode() if out else s


def _swap_tokens(rng, s: str, p: float = 0.1) -> str:
    if rng.random() >= p:
        return s
    w = s.split(" ")
    if len(w) < 2:
        return s
    i = int(rng.integers(0, len(w) - 1))
    w[i], w[i + 1] = w[i + 1], w[i]
    return " ".join(w)


@dataclass
class TablePair:
    left: List[List[str]]   # columns: id, title, authors, venue, year (no header)
    right: List[List[str]]
    true_pairs: np.ndarray  # (k, 2) data-row indices (header excluded)


HEADER = ["id", "title", "authors", "venue", "year"]


def make_tables(config: int, n_left: int, n_right: int, n_true: int, venues_left: Sequence[str],
                venue_draw_left, venue_draw_right, venues_right: Sequence[str], year_lo: int,
                year_hi: int, seed_offset: int = 0) -> TablePair:
    rng = np.random.Generator(np.random.PCG64(BASE_SEED + config + seed_offset))
    vocab = make_vocab(rng)
    lt = _titles(rng, vocab, n_left)
    la = _authors(rng, vocab, n_left)
    lv = [venues_left[i] for i in venue_draw_left(rng, n_left)]
    ly = [str(y) for y in rng.integers(year_lo, year_hi + 1, size=n_left)]
    n_rand = n_right - n_true
    rt = _titles(rng, vocab, n_rand)
    ra = _authors(rng, vocab, n_rand)
    rv = [venues_right[i] for i in venue_draw_right(rng, n_rand)]
    ry = [str(y) for y in rng.integers(year_lo, year_hi + 1, size=n_rand)]
    # only rng.integers / rng.random are used, whose streams numpy keeps stable
    if n_true <= n_left:
        src = np.argsort(rng.random(n_left), kind="stable")[:n_true]
    else:
        src = rng.integers(0, n_left, size=n_true)
    for i in src:
        rt.append(_swap_tokens(rng, _edit(rng, lt[i])))
        ra.append(_edit(rng, la[i]))
        rv.append(lv[i])
        ry.append(ly[i])
    perm = np.argsort(rng.random(n_right), kind="stable")
    rt = [rt[k] for k in perm]
    ra = [ra[k] for k in perm]
    rv = [rv[k] for k in perm]
    ry = [ry[k] for k in perm]
    inv = np.empty(n_right, dtype=np.int64)
    inv[perm] = np.arange(n_right)
    true_pairs = np.stack([src, inv[n_rand + np.arange(n_true)]], axis=1) if n_true else np.zeros((0, 2), np.int64)
    lid = [str(100000 + i) for i in range(n_left)]
    rid = [str(500000 + i) for i in range(n_right)]
    return TablePair([lid, lt, la, lv, ly], [rid, rt, ra, rv, ry], true_pairs)


def _q(s: str) -> str:
    return '"' + s.replace('"', '""') + '"'


def write_csv(path: str, cols: List[List[str]]) -> None:
    n = len(cols[0])
    with open(path, "w", newline="") as f:
        f.write(",".join(_q(h) for h in HEADER) + "\r\n")
        for i in range(n):
            f.write(f"{cols[0][i]},{_q(cols[1][i])},{_q(cols[2][i])},{_q(cols[3][i])},{cols[4][i]}\r\n")


def table_bytes(cols: List[List[str]]) -> List[List[bytes]]:
    """Column-major cells as the reference reads them: header row first."""
    return [[h.encode()] + [x.encode() for x in col] for h, col in zip(HEADER, cols)]


def rule_yaml(eq_cols: Sequence[int], sims: Sequence[tuple]) -> str:
    """A rule file in the reference's format (README.md example layout).

    sims: (column, threshold) pairs; both tables use the same column index.
    """
    eq = ", ".join(["0", "1"] + [f"{c}, {c}" for c in eq_cols])
    sim = ", ".join(["0", "1"] + [f"{c}, {c}" for c, _ in sims])
    thr = ", ".join(["0", "1"] + [f"{t}" for _, t in sims])
    return (
        "Preconditions:\n"
        "  Relations:\n"
        "    - [0, 0, 1, 2, 3, 4]\n"
        "    - [1, 0, 1, 2, 3, 4]\n"
        "  Equalities:\n"
        f"    - [{eq}]\n"
        "  Sim:\n"
        f"    - [{sim}]\n"
        "  Threshold:\n"
        f"    - [{thr}]\n"
        "Conseq:\n"
        "  Option:\n"
        "    Equality\n"
        "  Equality:\n"
        "    [0, 1, 0, 0]\n"
    )


@dataclass
class Workload:
    name: str
    tables: TablePair
    rules: List[str]           # YAML documents, written in this order
    n_partitions: int
    description: str = ""


def _venue_names(rng_seed: int, n: int) -> List[str]:
    rng = np.random.Generator(np.random.PCG64(rng_seed))
    w = _pseudo_words(rng, n * 3, 3, 9, cap=True)
    return [" ".join(w[3 * i:3 * i + 1 + (i % 3)]) + f" {i}" for i in range(n)]


def c1() -> Workload:
    """2,616 x 2,294 rows, 2,224 true pairs, 1 rule, 1 partition (DBLP-ACM shape)."""
    venues = _venue_names(BASE_SEED + 101, 5)
    uni = lambda rng, k: rng.integers(0, 5, size=k)
    t = make_tables(1, 2616, 2294, 2224, venues, uni, uni, venues, 1994, 2003)
    return Workload("c1_2616x2294_1rule_1part", t, [rule_yaml([4], [(1, 0.89), (2, 0.85)])], 1,
                    "year eq, JW(title)>=0.89, JW(authors)>=0.85")


def c2() -> Workload:
    """2,600 x 64,263 rows, 5k true pairs, 2 rules, 8 partitions."""
    venues = _venue_names(BASE_SEED + 102, 500)

    def vd(rng, k):
        w = 1.0 / np.arange(1, 501) ** 1.0
        cdf = np.cumsum(w) / w.sum()
        return np.minimum(np.searchsorted(cdf, rng.random(k), side="right"), 499)

    t = make_tables(2, 2600, 64263, 5000, venues, vd, vd, venues, 1980, 2005)
    rules = [rule_yaml([4], [(1, 0.89), (2, 0.85)]), rule_yaml([3], [(1, 0.95)])]
    return Workload("c2_2600x64263_2rules_8parts", t, rules, 8,
                    "(year eq, JW(title)>=0.89, JW(authors)>=0.85) or (venue eq, JW(title)>=0.95)")


WORKLOADS = {"c1": c1, "c2": c2}


def materialize(w: Workload, directory: str) -> Dict[str, str]:
    """Writes left.csv, right.csv and rules/<k>.yaml; returns the paths."""
    os.makedirs(directory, exist_ok=True)
    rd = os.path.join(directory, "rules")
    os.makedirs(rd, exist_ok=True)
    for f in os.listdir(rd):
        os.remove(os.path.join(rd, f))
    for k, doc in enumerate(w.rules):
        with open(os.path.join(rd, f"{k}.yaml"), "w") as f:
            f.write(doc)
    lp = os.path.join(directory, "left.csv")
    rp = os.path.join(directory, "right.csv")
    write_csv(lp, w.tables.left)
    write_csv(rp, w.tables.right)
    return {"left": lp, "right": rp, "rules": rd}
