"""Parity of the GPU engine with the oracle and the golden vectors.

Every test here calls the engine through its C ABI (libhbx.so via ctypes) on
the GPU and compares the set of (left row, right row) pairs bit-exactly with
the oracle (the reference's algorithm restated, brute force) on the same
seeded inputs, and with the golden digests made from the reference's own
kernel.  Both execution forms (plain per-partition launches and the batched
persistent launch) must give the identical set.
"""
import os
import subprocess

import numpy as np
import pytest

import hyperblocker_gb300 as hb
from oracle import api, csvref, rules
from hyperblocker_gb300 import synth
from tests import _util
from tests.golden.make_golden import edge_tables

pytestmark = pytest.mark.gpu

MODES = ["plain", "batched"]


def _oracle_plan(docs):
    return rules.serialize(rules.sort_rules([rules.decode_rule(rules.parse_yaml(d)) for d in docs]))


def _engine_pairs(ctx, docs, cl, cr, n_part, prefix=_util.INT_MAX, mode="batched"):
    plan = hb.Plan.from_yaml(docs, ctx)
    L = hb.Table.from_columns(cl, ctx)
    R = hb.Table.from_columns(cr, ctx)
    pairs, st = hb.block(ctx, plan, L, R, n_part, prefix, mode)
    return _util.sorted_pairs(pairs), st


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("case", ["edge_title_authors", "edge_title_only_no_eq",
                                  "edge_two_rules_3parts", "edge_prefix_hash", "edge_eq_only",
                                  "edge_threshold_one"])
def test_edge_cases(ctx, golden, case, mode):
    g = golden[case]
    el, er = edge_tables()
    pairs, st = _engine_pairs(ctx, g["rules"], el, er, g["n_partitions"], g["prefix_idx"], mode)
    lines = _util.id_lines(pairs, el, er)
    assert [[a.decode(), b.decode()] for a, b in lines] == g["pairs"]
    assert st.fma_ambiguous == 0


@pytest.mark.parametrize("mode", MODES)
def test_c1_csv_path(ctx, golden, tmp_path, mode):
    """C1 shape through the CSV reader and the rule directory, as the CLI runs."""
    w, paths, order = _util.materialize("c1", str(tmp_path))
    plan = hb.Plan.from_rule_dir(paths["rules"], ctx)
    L = hb.Table.from_csv(paths["left"], ",", ctx)
    R = hb.Table.from_csv(paths["right"], ",", ctx)
    pairs, st = hb.block(ctx, plan, L, R, w.n_partitions, _util.INT_MAX, mode)
    cl = csvref.read_columns(paths["left"])
    cr = csvref.read_columns(paths["right"])
    lines = _util.id_lines(pairs, cl, cr)
    g = golden["c1_order_0"]
    assert len(lines) == g["count"]
    assert _util.digest(lines) == g["sha256"]
    assert st.pair_comparisons == g["pair_comparisons"]
    assert st.pairs_covered == g["pairs_covered"]
    assert st.fma_ambiguous == 0


@pytest.mark.parametrize("mode", MODES)
def test_c2_against_oracle_and_golden(ctx, golden, tmp_path, mode):
    w, paths, order = _util.materialize("c2", str(tmp_path))
    plan = hb.Plan.from_rule_dir(paths["rules"], ctx)
    L = hb.Table.from_csv(paths["left"], ",", ctx)
    R = hb.Table.from_csv(paths["right"], ",", ctx)
    pairs, st = hb.block(ctx, plan, L, R, w.n_partitions, _util.INT_MAX, mode)
    cl = csvref.read_columns(paths["left"])
    cr = csvref.read_columns(paths["right"])
    g = golden["c2_order_" + "".join(map(str, order))]
    lines = _util.id_lines(pairs, cl, cr)
    assert len(lines) == g["count"]
    assert _util.digest(lines) == g["sha256"]
    assert st.pair_comparisons == g["pair_comparisons"]
    # and against the oracle run here on the very same directory
    res = api.run_block(api.CTable(cl), api.CTable(cr), rules.plan_from_dir(paths["rules"]),
                        w.n_partitions)
    assert np.array_equal(_util.sorted_pairs(pairs), res.pairs)


@pytest.mark.parametrize("seed", range(8))
def test_random_tables_against_oracle(ctx, seed):
    """Tiny alphabets, empty strings, strings past 64/128/256 bytes, several
    rules that overlap (cross-rule duplicates), 1-5 partitions, prefix hash."""
    alpha = [b"ab", b"abc", b"abcdefgh ", b"xyz, ", b"abcdefghijklmnopqrstuvwxyz"][seed % 5]
    max_len = [20, 70, 140, 300, 40, 260, 33, 64][seed]
    cl, cr = _util.random_tables(100 + seed, 50 + 7 * seed, 90, alpha, max_len)
    docs = [synth.rule_yaml([3], [(1, 0.72 + 0.02 * seed)]),
            synth.rule_yaml([4], [(2, 0.6), (1, 0.55)]),
            synth.rule_yaml([3, 4], [(2, 0.5)])]
    prefix = 1 if seed % 4 == 3 else _util.INT_MAX
    n_part = 1 + seed % 5
    want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), n_part, prefix)
    for mode in MODES:
        got, st = _engine_pairs(ctx, docs, cl, cr, n_part, prefix, mode)
        assert np.array_equal(got, want.pairs), mode
        assert st.pair_comparisons == want.pair_comparisons
        assert st.pairs_covered == want.pairs_covered


RULE_GROUP_SETS = [
    # one group over k1 (title first): the root, a member with the same
    # equalities (title and authors), two members with the extra equality k2,
    # each at its own title threshold; k2 alone roots a second group
    [synth.rule_yaml([3], [(1, 0.70)]), synth.rule_yaml([3, 4], [(1, 0.62), (2, 0.5)]),
     synth.rule_yaml([4, 3], [(2, 0.55), (1, 0.66)]), synth.rule_yaml([3], [(2, 0.7), (1, 0.8)]),
     synth.rule_yaml([4], [(1, 0.75)])],
    # the root tests authors before title; title is what its members share,
    # so it moves to the front of the group
    [synth.rule_yaml([3], [(2, 0.6), (1, 0.7)]), synth.rule_yaml([3, 4], [(1, 0.65)]),
     synth.rule_yaml([4, 3], [(1, 0.72), (2, 0.58)])],
    # no equalities at the root: every pair of a partition is a candidate
    [synth.rule_yaml([], [(1, 0.8)]), synth.rule_yaml([3], [(1, 0.7), (2, 0.6)]),
     synth.rule_yaml([4], [(1, 0.68)]), synth.rule_yaml([3, 4], [(2, 0.5), (1, 0.6)])],
]


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("rule_set", range(len(RULE_GROUP_SETS)))
def test_rule_groups_against_oracle(ctx, rule_set, seed):
    """The batched form evaluates rules whose equalities contain another
    rule's, and that test its first similarity column, inside that rule's
    join (one first-column scan per pair, decided per member); the plain form
    evaluates every rule on its own.  Both must give the oracle's set and
    pair-comparison count (every rule's candidates are still counted)."""
    alpha = [b"abc", b"abcdefgh ", b"xyz, ", b"abcdefghijklmnopqrstuvwxyz"][seed]
    cl, cr = _util.random_tables(500 + 10 * rule_set + seed, 70, 160, alpha, [30, 90, 140, 70][seed])
    docs = RULE_GROUP_SETS[rule_set]
    n_part = 1 + seed % 3
    want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), n_part)
    assert len(want.pairs) > 0
    for mode in MODES:
        got, st = _engine_pairs(ctx, docs, cl, cr, n_part, _util.INT_MAX, mode)
        assert np.array_equal(got, want.pairs), mode
        assert st.pair_comparisons == want.pair_comparisons, mode
        assert st.fma_ambiguous == 0


def _rule8(eq_cols, sims):
    """synth.rule_yaml over tables of 8 columns (id, s1, s2, k1, ..., k5)."""
    return synth.rule_yaml(eq_cols, sims).replace("[0, 0, 1, 2, 3, 4]", "[0, 0, 1, 2, 3, 4, 5, 6, 7]") \
        .replace("[1, 0, 1, 2, 3, 4]", "[1, 0, 1, 2, 3, 4, 5, 6, 7]")


def _tables8(seed):
    """random_tables plus three more equality columns k3, k4, k5 (2-3 values each)."""
    cl, cr = _util.random_tables(seed, 90, 200, b"abcdefgh ", 60, n_eq_values=2)
    rng = np.random.Generator(np.random.PCG64(seed + 7))

    def more(t, n):
        for name, k in ((b"k3", 2), (b"k4", 3), (b"k5", 2)):
            t.append([name] + [str(int(x)).encode() for x in rng.integers(0, k, size=n)])
        return t

    return more(cl, 90), more(cr, 200)


# groups whose members add extra equality slots: exactly two slots in all
# (the members' live set is looked up per pattern of slots that hold), and
# four (walked member by member)
EXTRA_SLOT_SETS = [
    [_rule8([3], [(1, 0.70)]), _rule8([3, 4], [(1, 0.62), (2, 0.5)]), _rule8([3, 5], [(1, 0.66)]),
     _rule8([3, 4, 5], [(1, 0.6)])],
    [_rule8([3], [(1, 0.70)]), _rule8([3, 4, 5], [(1, 0.62)]), _rule8([3, 6, 7], [(1, 0.66), (2, 0.55)]),
     _rule8([3, 4, 5, 6, 7], [(1, 0.6)])],
]


@pytest.mark.parametrize("seed", range(3))
@pytest.mark.parametrize("rule_set", range(len(EXTRA_SLOT_SETS)))
def test_rule_groups_with_extra_slots_against_oracle(ctx, rule_set, seed):
    """Group members with one to four extra equality slots: both forms give
    the oracle's set and pair-comparison count."""
    cl, cr = _tables8(900 + 10 * rule_set + seed)
    docs = EXTRA_SLOT_SETS[rule_set]
    n_part = 1 + seed
    want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), n_part)
    assert len(want.pairs) > 0
    for mode in MODES:
        got, st = _engine_pairs(ctx, docs, cl, cr, n_part, _util.INT_MAX, mode)
        assert np.array_equal(got, want.pairs), mode
        assert st.pair_comparisons == want.pair_comparisons, mode


@pytest.mark.parametrize("thr", ["nan", "inf", "-inf", "0x1.8p-1"])
def test_thresholds_stof_reads_besides_decimals(ctx, thr):
    """A threshold of nan never fails a pair (JW < nan is false in the
    reference, global_func.cuh:144), inf always does, -inf never; hexadecimal
    floats are numbers.  Alone and in a rule group, both forms agree with the
    oracle."""
    cl, cr = _util.random_tables(77, 60, 120, b"abcdef ", 40, n_eq_values=2)
    odd = synth.rule_yaml([3, 4], [(1, 0.5), (2, 0.6)]).replace("0.5, 0.6", f"{thr}, 0.6")
    for docs in ([odd], [synth.rule_yaml([3], [(1, 0.7)]), odd]):
        want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), 2)
        for mode in MODES:
            got, st = _engine_pairs(ctx, docs, cl, cr, 2, _util.INT_MAX, mode)
            assert np.array_equal(got, want.pairs), (thr, len(docs), mode)
            assert st.pair_comparisons == want.pair_comparisons


def test_planner_puts_the_selective_predicate_first(built):
    """The reference evaluates a rule's similarity predicates in YAML order
    (execution_plan_generator.h:111-137; its Prioritizer, :223, is declared
    and never defined).  Here the first predicate passes every pair
    (threshold 0: every candidate needs a scan) and the second almost none;
    the planner's measured order (hbx_opts.pred_order = 0) runs the selective
    one first, so far fewer pairs reach a scan than in YAML order
    (pred_order = 1), and the pairs are the same."""
    cl, cr = _util.random_tables(808, 300, 600, b"abcdefghij ", 40, n_eq_values=2)
    docs = [synth.rule_yaml([3], [(2, 0.0), (1, 0.97)])]
    want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), 1)
    scanned = {}
    for order in (0, 1):
        c = hb.Context(0, pred_order=order)
        plan = hb.Plan.from_yaml(docs, c)
        L = hb.Table.from_columns(cl, c)
        R = hb.Table.from_columns(cr, c)
        got, st = hb.block(c, plan, L, R, 1, _util.INT_MAX, "batched")
        assert np.array_equal(_util.sorted_pairs(got), want.pairs), order
        scanned[order] = st.pairs_scanned
        c.close()
    assert scanned[1] >= st.pair_comparisons // 2  # YAML order: the threshold-0 scan of every pair
    assert scanned[0] * 10 < scanned[1]


@pytest.mark.parametrize("n_values", [500, 1500, 3000, 40000])
def test_key_domains_across_scan_chunks(ctx, n_values):
    """Left key domains (2 partitions x codes x 5 length classes) of 3, 8
    and 15 scan chunks (chunk totals, then each chunk's scan) and beyond the
    fused join's limit (per-rule join kernels); one-chunk domains are the
    other tests' tables."""
    cl, cr = _util.random_tables(7000 + n_values, 2000, 100_000, b"abc", 12, n_eq_values=n_values)
    docs = [synth.rule_yaml([3], [(1, 0.6)]), synth.rule_yaml([3, 4], [(2, 0.7)])]
    want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), 2, _util.INT_MAX)
    assert len(want.pairs) > 100
    for mode in MODES:
        got, st = _engine_pairs(ctx, docs, cl, cr, 2, _util.INT_MAX, mode)
        assert np.array_equal(got, want.pairs), mode
        assert st.pair_comparisons == want.pair_comparisons
        assert st.pairs_covered == want.pairs_covered


def test_session_reuse_and_modes_agree(ctx, tmp_path):
    w, paths, _ = _util.materialize("c1", str(tmp_path))
    plan = hb.Plan.from_rule_dir(paths["rules"], ctx)
    L = hb.Table.from_csv(paths["left"], ",", ctx)
    R = hb.Table.from_csv(paths["right"], ",", ctx)
    import torch

    s = hb.Session(ctx, plan, L, R, w.n_partitions)
    cap = 1 << 16
    ol = torch.empty(cap, dtype=torch.int32, device="cuda")
    orr = torch.empty(cap, dtype=torch.int32, device="cuda")
    results = []
    for mode in ["batched", "batched", "plain", "batched"]:
        n = s.run_device(mode, ol.data_ptr(), orr.data_ptr(), cap)
        p = np.stack([ol[:n].cpu().numpy().view(np.uint32), orr[:n].cpu().numpy().view(np.uint32)], 1)
        results.append(_util.sorted_pairs(p))
    for r in results[1:]:
        assert np.array_equal(r, results[0])
    # too small a device buffer: CAPACITY with the required count, nothing reported written
    with pytest.raises(hb.HbxError) as e:
        s.run_device("batched", ol.data_ptr(), orr.data_ptr(), 3)
    assert e.value.status == hb.ERR_CAPACITY
    s.close()


def test_watchdog_budget_reports_and_context_survives(built, tmp_path):
    """A one-cycle budget stops the persistent loop: the call returns
    HBX_ERR_WATCHDOG (no hang, no fault) and the context keeps working."""
    w, paths, _ = _util.materialize("c1", str(tmp_path))
    c = hb.Context(0, watchdog_cycles=1)
    plan = hb.Plan.from_rule_dir(paths["rules"], c)
    L = hb.Table.from_csv(paths["left"], ",", c)
    R = hb.Table.from_csv(paths["right"], ",", c)
    with pytest.raises(hb.HbxError) as e:
        hb.block(c, plan, L, R, 1, _util.INT_MAX, "batched")
    assert e.value.status == hb.ERR_WATCHDOG
    c.close()
    c2 = hb.Context(0)
    pairs, _ = hb.block(c2, plan, L, R, 1, _util.INT_MAX, "batched")
    assert len(pairs) > 0
    c2.close()


def test_cli_drop_in(built, golden, tmp_path):
    """run_hyperblocker_exec with the reference's flags appends id pairs."""
    w, paths, _ = _util.materialize("c1", str(tmp_path))
    out = str(tmp_path / "pairs.csv")
    cmd = [hb.EXE_PATH, "-data_l", paths["left"], "-data_r", paths["right"], "-rule_dir",
           paths["rules"], "-n_partitions", "1", "-o", out, "-scheduler=CHBL"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = open(out, "rb").read().splitlines()
    pairs = sorted(tuple(x.split(b",", 1)) for x in lines)
    assert _util.digest(pairs) == golden["c1_order_0"]["sha256"]
    r = subprocess.run(cmd + ["-hbx_mode=plain"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert len(open(out, "rb").read().splitlines()) == 2 * len(lines)  # append mode


def test_reference_class_shape_writes_what_the_cli_writes(built, golden, tmp_path):
    """hb.HyperBlocker(rule_dir, data_l, data_r, output, n_partitions).Run(),
    the reference's class (core/hyperblocker.cuh:45-131), appends the same
    lines as run_hyperblocker_exec: the golden pair set, in row order."""
    w, paths, _ = _util.materialize("c1", str(tmp_path))
    out_cls, out_cli = str(tmp_path / "cls.csv"), str(tmp_path / "cli.csv")
    pairs = hb.HyperBlocker(paths["rules"], paths["left"], paths["right"], out_cls, 1).Run()
    assert len(pairs) > 0
    cmd = [hb.EXE_PATH, "-data_l", paths["left"], "-data_r", paths["right"], "-rule_dir",
           paths["rules"], "-n_partitions", "1", "-o", out_cli]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = open(out_cls, "rb").read()
    assert got == open(out_cli, "rb").read()
    lines = sorted(tuple(x.split(b",", 1)) for x in got.splitlines())
    assert _util.digest(lines) == golden["c1_order_0"]["sha256"]


@pytest.mark.parametrize("tile", [32, 64, 128])
@pytest.mark.parametrize("variant", [1, 2])
def test_tile_shapes_and_kernel_variants_agree(built, tile, variant):
    """Every tile shape and both evaluation kernels give the oracle's pairs."""
    cl, cr = _util.random_tables(500 + tile, 80, 400, b"abcdefgh ,", 150)
    docs = [synth.rule_yaml([3], [(1, 0.7)]), synth.rule_yaml([4], [(2, 0.6), (1, 0.5)])]
    want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), 2)
    c = hb.Context(0, tile_right=tile, eval_variant=variant)
    for mode in MODES:
        got, st = _engine_pairs(c, docs, cl, cr, 2, _util.INT_MAX, mode)
        assert np.array_equal(got, want.pairs), (tile, variant, mode)
    c.close()


@pytest.mark.parametrize("variant", [1, 2])
def test_pairs_of_many_items_share_a_warp(built, variant):
    """A warp's lanes scan pairs of different work items, rules and
    predicates at once: an equality-only rule (emitted at claim time) beside
    rules of one and two predicates over strings of 0-300 bytes (every scan
    width, tables and the reference loops in one launch), many small
    candidate blocks, every tile shape."""
    cl, cr = _util.random_tables(911, 300, 700, b"abcde ", 300, n_eq_values=40)
    docs = [synth.rule_yaml([3, 4], []),
            synth.rule_yaml([3], [(1, 0.62)]),
            synth.rule_yaml([4], [(2, 0.58), (1, 0.52)])]
    want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), 3)
    for tile in (32, 64, 128):
        c = hb.Context(0, tile_right=tile, eval_variant=variant)
        for mode in MODES:
            got, st = _engine_pairs(c, docs, cl, cr, 3, _util.INT_MAX, mode)
            assert np.array_equal(got, want.pairs), (tile, mode)
            assert st.pair_comparisons == want.pair_comparisons
            assert st.fma_ambiguous == 0
        c.close()


def test_string_lengths_at_word_and_table_boundaries(ctx):
    """Left and right strings of 0-300 bytes around every scan-width and
    table boundary (32, 64, 96, 128, 256 = the longest string with a Peq
    table), over a 3-symbol alphabet so that many pairs reach a scan, on both
    predicates of a rule (the second one reached only by pairs that pass the
    first)."""
    lens = [0, 1, 2, 15, 16, 17, 31, 32, 33, 63, 64, 65, 95, 96, 97, 127, 128, 129, 160,
            255, 256, 257, 300]
    rng = np.random.Generator(np.random.PCG64(2024))

    def table(n, prefix):
        def s():
            return bytes(rng.choice(list(b"abc"), size=lens[int(rng.integers(0, len(lens)))]).tolist())
        ids = [b"id"] + [f"{prefix}{i}".encode() for i in range(n)]
        return [ids, [b"s1"] + [s() for _ in range(n)], [b"s2"] + [s() for _ in range(n)],
                [b"k1"] + [b"0"] * n, [b"k2"] + [b"0"] * n]

    cl, cr = table(120, "l"), table(160, "r")
    docs = [synth.rule_yaml([3], [(1, 0.62), (2, 0.6)])]
    want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), 1)
    for mode in MODES:
        got, st = _engine_pairs(ctx, docs, cl, cr, 1, _util.INT_MAX, mode)
        assert np.array_equal(got, want.pairs), mode
        assert st.fma_ambiguous == 0
    assert len(want.pairs) > 100


def test_autotuner_choice_is_cached_and_exact(built, tmp_path, monkeypatch):
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("HBX_AUTOTUNE_CACHE", str(cache))
    cl, cr = _util.random_tables(77, 200, 600, b"abcdefgh ,", 90)
    docs = [synth.rule_yaml([3], [(1, 0.7)])]
    want = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), 1)
    for _ in range(2):  # first run tunes and writes the cache, second reads it
        c = hb.Context(0)
        got, _ = _engine_pairs(c, docs, cl, cr, 1)
        assert np.array_equal(got, want.pairs)
        c.close()
    text = cache.read_text()
    assert text.startswith("{") and "|L" in text
