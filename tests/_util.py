"""Shared helpers of the test suite (not collected: no test_ prefix)."""
from __future__ import annotations

import hashlib
import os
from typing import List, Sequence, Tuple

import numpy as np

from hyperblocker_gb300 import synth

INT_MAX = 2147483647


def digest(lines: Sequence[Tuple[bytes, bytes]]) -> str:
    h = hashlib.sha256()
    for a, b in lines:
        h.update(a + b"," + b + b"\n")
    return h.hexdigest()


def id_lines(pairs: np.ndarray, cols_l, cols_r) -> List[Tuple[bytes, bytes]]:
    return sorted((cols_l[0][int(l)], cols_r[0][int(r)]) for l, r in pairs)


def sorted_pairs(pairs: np.ndarray) -> np.ndarray:
    if len(pairs) == 0:
        return np.zeros((0, 2), dtype=np.uint32)
    p = np.asarray(pairs, dtype=np.uint32)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def materialize(name: str, directory: str):
    """Writes a synthetic workload; returns (workload, paths, rule order as read)."""
    w = synth.WORKLOADS[name]()
    paths = synth.materialize(w, directory)
    order = [int(e.name.split(".")[0]) for e in os.scandir(paths["rules"])]
    return w, paths, order


def random_tables(seed: int, n_l: int, n_r: int, alphabet: bytes, max_len: int,
                  n_eq_values: int = 3):
    """Small random tables: id, s1, s2, k1, k2 (header row first)."""
    rng = np.random.Generator(np.random.PCG64(seed))

    def strings(n):
        out = []
        for _ in range(n):
            L = int(rng.integers(0, max_len + 1)) if rng.random() > 0.05 else 0
            out.append(bytes(alphabet[int(i)] for i in rng.integers(0, len(alphabet), size=L)))
        return out

    def table(n, prefix):
        ids = [b"id"] + [f"{prefix}{i}".encode() for i in range(n)]
        s1 = [b"s1"] + strings(n)
        s2 = [b"s2"] + strings(n)
        k1 = [b"k1"] + [str(int(x)).encode() for x in rng.integers(0, n_eq_values, size=n)]
        k2 = [b"k2"] + [str(int(x)).encode() for x in rng.integers(0, 2, size=n)]
        return [ids, s1, s2, k1, k2]

    return table(n_l, "l"), table(n_r, "r")
