"""The oracle, pinned: against the golden vectors made from the reference's own
kernel, against the reference kernel itself where it is built, and the
algorithmic fact the GPU kernel relies on (bit-parallel maximum matching ==
the reference's Jaro loops).  No GPU needed."""
import os
import random

import numpy as np
import pytest

from oracle import api, csvref, rules
from hyperblocker_gb300 import synth
from tests import _util
from tests.golden.make_golden import edge_tables

REF_DATA = os.path.join(api.REFERENCE_ROOT, "data", "dblp-acm")


@pytest.fixture(scope="module", autouse=True)
def _built():
    api.build()


def _plan(docs):
    return rules.serialize(rules.sort_rules([rules.decode_rule(rules.parse_yaml(d)) for d in docs]))


@pytest.mark.skipif(not os.path.isdir(REF_DATA), reason="reference checkout not mounted")
@pytest.mark.parametrize("thr,count,tp", [("0.89, 0.85", 1995, 1922), ("0.81, 0.79", 2477, 2099)])
def test_dblp_acm_known_answers(golden, thr, count, tp):
    A = csvref.read_columns(os.path.join(REF_DATA, "tableA.csv"))
    B = csvref.read_columns(os.path.join(REF_DATA, "tableB.csv"))
    M = csvref.read_columns(os.path.join(REF_DATA, "match.csv"))
    src = open(os.path.join(REF_DATA, "rules", "0.yaml")).read().replace("0.81, 0.79", thr)
    res = api.run_block(api.CTable(A), api.CTable(B), _plan([src]), 1)
    lines = _util.id_lines(res.pairs, A, B)
    g = golden[f"dblp_acm_{thr.replace(', ', '_')}"]
    assert len(lines) == count == g["count"]
    assert len(set(lines) & set(zip(M[0], M[1]))) == tp == g["true_positives"]
    assert _util.digest(lines) == g["sha256"]
    assert res.fma_ambiguous == 0


@pytest.mark.parametrize("case", ["c1_order_0", "c2_order_01", "c2_order_10"])
def test_synthetic_golden(golden, case):
    g = golden[case]
    w = synth.WORKLOADS[g["workload"]]()
    cl, cr = synth.table_bytes(w.tables.left), synth.table_bytes(w.tables.right)
    import hashlib

    assert hashlib.sha256(b"\0".join(b"\1".join(c) for c in cl)).hexdigest() == g["left_sha256"]
    assert hashlib.sha256(b"\0".join(b"\1".join(c) for c in cr)).hexdigest() == g["right_sha256"]
    plan = _plan([w.rules[k] for k in g["rule_order"]])
    res = api.run_block(api.CTable(cl), api.CTable(cr), plan, g["n_partitions"])
    lines = _util.id_lines(res.pairs, cl, cr)
    assert len(lines) == g["count"]
    assert _util.digest(lines) == g["sha256"]
    assert res.pair_comparisons == g["pair_comparisons"]
    assert res.pairs_covered == g["pairs_covered"]


@pytest.mark.parametrize("case", ["edge_title_authors", "edge_title_only_no_eq",
                                  "edge_two_rules_3parts", "edge_prefix_hash", "edge_eq_only",
                                  "edge_threshold_one"])
def test_edge_golden(golden, case):
    g = golden[case]
    el, er = edge_tables()
    res = api.run_block(api.CTable(el), api.CTable(er), _plan(g["rules"]), g["n_partitions"],
                        g["prefix_idx"])
    lines = _util.id_lines(res.pairs, el, er)
    assert [[a.decode(), b.decode()] for a, b in lines] == g["pairs"]
    assert _util.digest(lines) == g["sha256"]


@pytest.mark.skipif(not api.ref_available(), reason="reference kernel not built here")
@pytest.mark.parametrize("seed", range(6))
def test_port_equals_reference_kernel(seed):
    """Random small tables, tiny alphabets, strings up to 300 bytes."""
    alpha = [b"ab", b"abc", b"abcdefgh ", b"xyz, "][seed % 4]
    cl, cr = _util.random_tables(seed, 40, 60, alpha, 300 if seed % 3 == 0 else 40)
    docs = [synth.rule_yaml([3], [(1, 0.7 + 0.03 * seed)]),
            synth.rule_yaml([4], [(2, 0.6), (1, 0.5)])]
    plan = _plan(docs)
    for n_part in (1, 3):
        L, R = api.CTable(cl), api.CTable(cr)
        ref = api.run_ref_block(L, R, plan, n_part)
        port = api.run_block(L, R, plan, n_part)
        assert _util.id_lines(port.pairs, cl, cr) == ref


def _jaro_from_m(m, ls, ll):
    if ls == 0 or ll == 0:
        return 1.0 if ls == ll else 0.0
    if m == 0:
        return 0.0
    md = np.float32(m)
    q = np.float32(np.float32(md / np.float32(ls)) + np.float32(md / np.float32(ll)))
    return float(np.float32((float(q) + 1.0) / 3.0))


def _m_bitparallel(a: bytes, b: bytes) -> int:
    """The GPU kernel's algorithm: Peq of a, greedy over b, lowest free bit."""
    la, lb = len(a), len(b)
    if not la or not lb:
        return 0
    h = (min(la, lb) + 1) // 2
    peq = {}
    for j, c in enumerate(a):
        peq[c] = peq.get(c, 0) | (1 << j)
    matched, win = 0, (1 << (h + 1)) - 1
    for i in range(min(lb, la + h)):
        x = peq.get(b[i], 0) & win & ~matched
        matched |= x & -x
        win = (win << 1) | (1 if i + 1 <= h else 0)
    return bin(matched).count("1")


def test_bitparallel_equals_reference_loops():
    L = api.lib()
    rnd = random.Random(7)
    for t in range(20000):
        alpha = rnd.choice([b"ab", b"abc", b"abcd", b"abcdefgh", b"abcdefghijklmnopqrstuvwxyz "])
        la = rnd.randint(0, 40 if t % 10 else 256)
        lb = rnd.randint(0, 40 if t % 10 else 300)
        if t % 3 == 0:
            lb = la
        a = bytes(rnd.choice(alpha) for _ in range(la))
        b = bytes(rnd.choice(alpha) for _ in range(lb))
        ref = np.float32(L.hbo_jaro(a, la, b, lb))
        for x, y in ((a, b), (b, a)):
            if len(x) > 256:
                continue
            got = np.float32(_jaro_from_m(_m_bitparallel(x, y), min(la, lb), max(la, lb)))
            assert got == ref, (a, b)


def test_jw_formula_details():
    L = api.lib()
    # uncapped prefix: 10 shared leading characters force 1.0
    assert L.hbo_jw(b"abcdefghijXYZ", 13, b"abcdefghijQRSTUV", 16, 1) == 1.0
    # both empty -> 1.0, one empty -> 0.0
    assert L.hbo_jw(b"", 0, b"", 0, 1) == 1.0
    assert L.hbo_jw(b"", 0, b"abc", 3, 1) == 0.0
    # transpositions are ignored: jaro of "ab" vs "ba" is 1.0 here
    assert L.hbo_jaro(b"ab", 2, b"ba", 2) == 1.0
    # the reference's window uses the shorter length: h = (min + 1) / 2
    assert abs(L.hbo_jaro(b"martha", 6, b"marhta", 6) - 1.0) < 1e-7


def test_partition_uses_std_hash():
    """Bucket = std::hash<std::string>(cell) % n on plan slot 0's column."""
    L = api.lib()
    cols = [[b"id", b"1", b"2"], [b"t", b"x", b"y"], [b"a", b"p", b"q"], [b"v", b"m", b"n"],
            [b"year", b"1999", b"2000"]]
    plan = _plan([synth.rule_yaml([4], [(1, 0.5)])])
    b = api.partition(api.CTable(cols), plan, 7)
    for i, cell in enumerate(cols[4]):
        assert b[i] == L.hbo_std_hash(cell, len(cell)) % 7


def _jw_fp64_py(a: bytes, b: bytes) -> float:
    """FP64 Jaro-Winkler from the bit-parallel match count: no float rounding."""
    la, lb = len(a), len(b)
    if la == 0 or lb == 0:
        j = 1.0 if la == lb else 0.0
    else:
        x, y = (a, b) if la <= lb else (b, a)
        m = _m_bitparallel(x, y)
        j = 0.0 if m == 0 else (m / min(la, lb) + m / max(la, lb) + 1.0) / 3.0
    p = 0
    while p < min(la, lb) and a[p] == b[p]:
        p += 1
    return min(1.0, j + (1.0 - j) * p * 0.1)


def test_fp64_restatement_and_its_distance():
    """hbo_jw_fp64 is the double-only formula over the reference's match
    count and prefix; the reference's float/double value lies within float
    rounding of it (the report's max |JW_fp32path - JW_fp64|)."""
    L = api.lib()
    rnd = random.Random(11)
    worst = 0.0
    for t in range(5000):
        alpha = rnd.choice([b"ab", b"abcd", b"abcdefghijklmnopqrstuvwxyz "])
        la, lb = rnd.randint(0, 60), rnd.randint(0, 60)
        a = bytes(rnd.choice(alpha) for _ in range(la))
        b = bytes(rnd.choice(alpha) for _ in range(lb))
        wide = L.hbo_jw_fp64(a, la, b, lb)
        assert abs(wide - _jw_fp64_py(a, b)) < 1e-12, (a, b)
        worst = max(worst, abs(L.hbo_jw(a, la, b, lb, 1) - wide))
    assert 0.0 < worst < 1e-6


def test_fp64_report_on_c2(golden):
    """Every JW evaluation of the C2 golden run is also evaluated in FP64: the
    report counts them, the decisions that FP64 would flip (none on C2) and
    the largest score difference; the reference path's set is unchanged."""
    g = golden["c2_order_01"]
    w = synth.WORKLOADS[g["workload"]]()
    cl, cr = synth.table_bytes(w.tables.left), synth.table_bytes(w.tables.right)
    res = api.run_block(api.CTable(cl), api.CTable(cr),
                        _plan([w.rules[k] for k in g["rule_order"]]), g["n_partitions"])
    assert _util.digest(_util.id_lines(res.pairs, cl, cr)) == g["sha256"]
    assert res.jw_evals > g["pair_comparisons"] // 2
    assert res.fp64_flips == 0
    assert 0.0 < res.fp64_max_abs_diff < 1e-6


def test_blob_tables_equal_cell_tables():
    """The oracle reads (blob, offsets) columns in place: same result as
    per-cell bytes (the form the 1M-10M-row checks use)."""
    cl, cr = _util.random_tables(5, 80, 120, b"abcdef ,", 30)

    def blobs(cols):
        out = []
        for col in cols:
            off = np.zeros(len(col) + 1, dtype=np.int64)
            off[1:] = np.cumsum([len(x) for x in col])
            out.append((np.frombuffer(b"".join(col) or b"\0", dtype=np.uint8), off))
        return out

    plan = _plan([synth.rule_yaml([3], [(1, 0.6)]), synth.rule_yaml([4], [(2, 0.5)])])
    a = api.run_block(api.CTable(cl), api.CTable(cr), plan, 3)
    b = api.run_block(api.CTable(blobs(cl)), api.CTable(blobs(cr)), plan, 3)
    assert np.array_equal(a.pairs, b.pairs)
    assert (a.pair_comparisons, a.pairs_covered) == (b.pair_comparisons, b.pairs_covered)


def test_stof_restatement_matches_libc_strtof():
    """The reference reads thresholds with std::stof (yaml_config.h:45),
    which is strtof plus an exception when nothing converts or the value is
    out of range (ERANGE).  The oracle's restatement (oracle/rules.py _stof)
    agrees with this host's strtof on every form."""
    import ctypes
    import ctypes.util
    import math

    import numpy as np

    from oracle.rules import RuleError, _stof

    libc = ctypes.CDLL(ctypes.util.find_library("c"), use_errno=True)
    libc.strtof.restype = ctypes.c_float
    libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]

    def stof(s):
        b = s.encode()
        end = ctypes.c_char_p()
        ctypes.set_errno(0)
        v = libc.strtof(b, ctypes.byref(end))
        consumed = ctypes.cast(end, ctypes.c_void_p).value - ctypes.cast(ctypes.c_char_p(b), ctypes.c_void_p).value
        if consumed == 0 or ctypes.get_errno() == 34:  # no conversion, or ERANGE
            return None
        return float(np.float32(v))

    cases = ["0.85", "0.5", " 0.7", "\t.25", "+0.9", "-0.3", "1", "1.", "1e-1", "2.5E+0", "7e-1x",
             "0.95abc", "nan", "NaN", "-nan", "nan(123)", "inf", "-INF", "Infinity", "infinityx",
             "0x1.8p-1", "0X10", "0x.8", "0x1p+2", "3.4e38", "3.5e38", "1e400", "1e-50", "1e-38",
             "1.2e-38", "0", "0.0", "-0", "abc", "", " ", "e5", ".", "+", "0x"]
    rng = np.random.Generator(np.random.PCG64(11))
    cases += [f"{x:.{int(rng.integers(1, 9))}g}" for x in rng.random(300)]
    for s in cases:
        want = stof(s)
        try:
            got = _stof(s)
        except RuleError:
            got = None
        if want is None or got is None:
            assert want is None and got is None, (s, want, got)
        elif math.isnan(want):
            assert math.isnan(got), s
        else:
            assert got == want, (s, want, got)
