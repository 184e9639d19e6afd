"""Blocking in partition windows (hbx_block_streamed).

With any window budget -- one window, many windows, partitions split by their
left rows -- the pairs, pair comparisons and pairs covered equal hbx_block's
(and the oracle's) on the same inputs.
"""
import numpy as np
import pytest

import hyperblocker_gb300 as hb
from hyperblocker_gb300 import synth
from oracle import api, rules
from tests import _util

pytestmark = pytest.mark.gpu


def _oracle_plan(docs):
    return rules.serialize(rules.sort_rules([rules.decode_rule(rules.parse_yaml(d)) for d in docs]))


def _both(ctx, docs, cl, cr, n_part, budget, prefix=_util.INT_MAX, mode="batched"):
    plan = hb.Plan.from_yaml(docs, ctx)
    L = hb.Table.from_columns(cl, ctx)
    R = hb.Table.from_columns(cr, ctx)
    want, sw = hb.block(ctx, plan, L, R, n_part, prefix, mode)
    got, sg = hb.block_streamed(ctx, plan, L, R, n_part, budget, prefix, mode)
    return _util.sorted_pairs(want), sw, _util.sorted_pairs(got), sg


@pytest.mark.parametrize("budget", [1 << 30, 1 << 16, 4096])
@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_windows_equal_one_shot(ctx, budget, mode):
    cl, cr = _util.random_tables(41, 700, 1500, b"abcdef ", 40, n_eq_values=5)
    docs = [synth.rule_yaml([3], [(1, 0.6)]), synth.rule_yaml([4], [(2, 0.65)])]
    want, sw, got, sg = _both(ctx, docs, cl, cr, 7, budget, mode=mode)
    assert np.array_equal(got, want)
    assert sg.pair_comparisons == sw.pair_comparisons
    assert sg.pairs_covered == sw.pairs_covered
    assert sg.n_partitions_used == sw.n_partitions_used
    if budget == 4096:
        assert sg.n_windows > 7  # partitions split by their left rows
    if budget == 1 << 30:
        assert sg.n_windows == 1
    oracle = api.run_block(api.CTable(cl), api.CTable(cr), _oracle_plan(docs), 7)
    assert np.array_equal(got, oracle.pairs)


def test_windows_with_prefix_hash(ctx):
    cl, cr = _util.random_tables(42, 400, 900, b"abcxyz ", 30)
    docs = [synth.rule_yaml([3], [(1, 0.5)])]
    want, sw, got, sg = _both(ctx, docs, cl, cr, 5, 8192, prefix=1)
    assert np.array_equal(got, want)
    assert sg.n_windows > 1


def test_single_partition_split_by_left_rows(ctx):
    cl, cr = _util.random_tables(43, 600, 800, b"ab", 20)
    docs = [synth.rule_yaml([], [(1, 0.7)])]
    want, sw, got, sg = _both(ctx, docs, cl, cr, 1, 16384)
    assert np.array_equal(got, want)
    assert sg.n_windows > 1
