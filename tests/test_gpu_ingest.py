"""Device-side table encoding (hyperblocker_gb300/csrc/ingest.cu).

A session encodes its tables on the GPU by default: partition buckets with a
restatement of libstdc++'s std::hash (data_mngr.h:150-202), joint
dictionaries, the symbol alphabet, arenas and string metadata.  Every case
here runs the same inputs through the device encoder and the host encoder
(hbx_opts.ingest = 1) and requires both to give the oracle's pair set and
the same pairs_covered / pair_comparisons, including composite join keys
(built on the device) and dictionary hash collisions (rebuilt on the device
with another seed).
"""

import numpy as np
import pytest

import hyperblocker_gb300 as hb
from oracle import api, rules
from hyperblocker_gb300 import synth
from tests import _util

pytestmark = pytest.mark.gpu


def _oracle_plan(docs):
    return rules.serialize(rules.sort_rules([rules.decode_rule(rules.parse_yaml(d)) for d in docs]))


def _run(ingest, docs, cl, cr, n_part, prefix, mode):
    c = hb.Context(0, ingest=ingest)
    try:
        plan = hb.Plan.from_yaml(docs, c)
        L = hb.Table.from_columns(cl, c)
        R = hb.Table.from_columns(cr, c)
        pairs, st = hb.block(c, plan, L, R, n_part, prefix, mode)
        return _util.sorted_pairs(pairs), st
    finally:
        c.close()


def _check(docs, cl, cr, n_part, prefix=_util.INT_MAX, expect_device=True):
    want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), n_part, prefix)
    for mode in ("batched", "plain"):
        dev, sd = _run(0, docs, cl, cr, n_part, prefix, mode)
        host, sh = _run(1, docs, cl, cr, n_part, prefix, mode)
        assert sh.ingest_on_device == 0
        assert sd.ingest_on_device == (1 if expect_device else 0)
        assert np.array_equal(dev, want.pairs), mode
        assert np.array_equal(host, want.pairs), mode
        assert sd.pairs_covered == sh.pairs_covered == want.pairs_covered
        assert sd.pair_comparisons == sh.pair_comparisons == want.pair_comparisons
    return want


def _nul_tables(seed):
    """Cells with NUL bytes: equal up to the NUL (equalities_kernel) but hashed
    whole for the partition bucket (std::hash<std::string>)."""
    rng = np.random.Generator(np.random.PCG64(seed))

    def table(n, prefix):
        ids = [b"id"] + [f"{prefix}{i}".encode() for i in range(n)]
        s1, k1 = [b"s1"], [b"k1"]
        for _ in range(n):
            L = int(rng.integers(0, 30))
            s = bytes(b"ab\x00cd "[int(i)] for i in rng.integers(0, 6, size=L))
            s1.append(s)
            k1.append(str(int(rng.integers(0, 3))).encode() +
                      (b"\x00" + bytes([97 + int(rng.integers(0, 3))]) if rng.random() < 0.5 else b""))
        return [ids, s1, s1[:], k1, k1[:]]

    return table(300, "l"), table(500, "r")


def test_nul_bytes_in_cells(built):
    cl, cr = _nul_tables(5)
    docs = [synth.rule_yaml([3], [(1, 0.6)])]
    for n_part in (1, 7):
        _check(docs, cl, cr, n_part)


@pytest.mark.parametrize("n_part", [1, 3, 64, 5000])
def test_partition_counts(built, n_part):
    """5000 partitions counts buckets in global memory instead of shared."""
    cl, cr = _util.random_tables(31, 400, 900, b"abcdef ", 40, n_eq_values=50)
    docs = [synth.rule_yaml([3], [(1, 0.6)]), synth.rule_yaml([4], [(2, 0.7)])]
    _check(docs, cl, cr, n_part)


def test_prefix_hash(built):
    cl, cr = _util.random_tables(32, 300, 700, b"abcxyz ", 30)
    docs = [synth.rule_yaml([3], [(1, 0.5)])]
    _check(docs, cl, cr, 5, prefix=1)


def test_long_and_empty_strings(built):
    """Strings past 16 symbols (the metadata head), past 256 bytes (the exact
    per-lane path) and empty ones."""
    cl, cr = _util.random_tables(33, 150, 300, b"ab", 300)
    docs = [synth.rule_yaml([4], [(1, 0.55), (2, 0.5)])]
    _check(docs, cl, cr, 2)


def test_no_equalities(built):
    cl, cr = _util.random_tables(34, 120, 260, b"abcd", 25)
    docs = [synth.rule_yaml([], [(1, 0.8)])]
    _check(docs, cl, cr, 1)


def test_composite_keys_on_the_device(built):
    """Two equalities with ~4000 distinct values each: the mixed-radix key
    domain is above 2^24, so the join needs composite ids; the device encoder
    builds them (tuple dictionary, ids regrouped by partition) and gives the
    host encoder's pairs and counts."""
    rng = np.random.Generator(np.random.PCG64(35))

    def table(n, prefix):
        ids = [b"id"] + [f"{prefix}{i}".encode() for i in range(n)]
        s1 = [b"s1"] + [bytes(b"abc"[int(i)] for i in rng.integers(0, 3, size=8)) for _ in range(n)]
        k1 = [b"k1"] + [str(int(x)).encode() for x in rng.integers(0, 4000, size=n)]
        k2 = [b"k2"] + [str(int(x)).encode() for x in rng.integers(0, 4000, size=n)]
        return [ids, s1, s1[:], k1, k2]

    cl, cr = table(6000, "l"), table(6000, "r")
    # make some rows agree on both keys
    for i in range(1, 400):
        cr[3][i], cr[4][i] = cl[3][i], cl[4][i]
    docs = [synth.rule_yaml([3, 4], [(1, 0.5)]), synth.rule_yaml([3], [(1, 0.9)])]
    _check(docs, cl, cr, 2)


def test_dictionary_collisions_are_rebuilt_on_the_device(built, monkeypatch):
    """HBX_TEST_DICT_COLLIDE=1 makes the first dictionary build keep 3 bits of
    each hash, so distinct cells collide; the exact check against each slot's
    representative finds it and the dictionaries are rebuilt with the next
    seed, on the device, with the same result (composite keys included)."""
    monkeypatch.setenv("HBX_TEST_DICT_COLLIDE", "1")
    cl, cr = _util.random_tables(36, 150, 400, b"abcdef", 30, n_eq_values=40)
    docs = [synth.rule_yaml([3], [(1, 0.6)]), synth.rule_yaml([3, 4], [(2, 0.5)])]
    _check(docs, cl, cr, 3)


def test_c2_shape_device_and_host_agree(built, tmp_path):
    """The C2 workload through both encoders (CSV reader, rule directory)."""
    w, paths, _ = _util.materialize("c2", str(tmp_path))
    out = {}
    for ingest in (0, 1):
        c = hb.Context(0, ingest=ingest)
        plan = hb.Plan.from_rule_dir(paths["rules"], c)
        L = hb.Table.from_csv(paths["left"], ",", c)
        R = hb.Table.from_csv(paths["right"], ",", c)
        pairs, st = hb.block(c, plan, L, R, w.n_partitions, _util.INT_MAX, "batched")
        out[ingest] = (_util.sorted_pairs(pairs), st.pairs_covered, st.pair_comparisons,
                       st.ingest_on_device)
        c.close()
    assert out[0][3] == 1 and out[1][3] == 0
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1:3] == out[1][1:3]
