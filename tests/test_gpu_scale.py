"""Parity at the shapes the targets are quoted on, reduced to test size.

The large workloads cannot be checked pair for pair in full on the CPU, so
these tests take a stratified sample of left rows -- the same number from
every reference partition (core/components/data_mngr.h:121-216) -- and
require the engine's pairs of those rows to equal the oracle's exactly
(plan semantics: core/gpu/global_func.cuh:117-183).  The bench runs the same
checks at full size (1M x 1M C3, 500k C5 shape, 10M-row resident serving).
"""
import numpy as np
import pytest

import hyperblocker_gb300 as hb
from hyperblocker_gb300 import synth_big
from oracle import api, rules
from tests._util import sorted_pairs

pytestmark = pytest.mark.gpu


def _oracle_plan(docs):
    return rules.serialize(rules.sort_rules([rules.decode_rule(rules.parse_yaml(d)) for d in docs]))


def _stratified(ctable, plan_o, n_part, per_part, seed):
    bucket = api.partition(ctable, plan_o, n_part)
    rng = np.random.Generator(np.random.PCG64(seed))
    filt = np.zeros(ctable.n_rows, dtype=np.uint8)
    for p in range(n_part):
        rows = np.nonzero(bucket == p)[0]
        if len(rows):
            filt[rng.choice(rows, size=min(per_part, len(rows)), replace=False)] = 1
    return filt


def _rows_of(pairs, filt):
    pairs = sorted_pairs(pairs)
    return pairs[filt[pairs[:, 0]] == 1] if len(pairs) else pairs


@pytest.fixture(scope="module")
def c3_small():
    return synth_big.c3(100_000, 100_000, 2_000)


@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_c3_reduced_sampled_parity(built, ctx, c3_small, mode):
    """100k x 100k rows, the C3 rule set (8 rules, 1-2 equalities, 1-3 JW
    predicates) and 64 Zipf(1.3)-sized partitions; 32 left rows of every
    partition checked against the oracle."""
    w = c3_small
    plan = hb.Plan.from_yaml(w.rules, ctx)
    L = hb.Table.from_columns(w.left.cols, ctx)
    R = hb.Table.from_columns(w.right.cols, ctx)
    got, st = hb.block(ctx, plan, L, R, w.n_partitions, hb.INT_MAX, mode)
    assert st.fma_ambiguous == 0
    assert st.n_partitions_used > 32  # the Zipf key spreads over most partitions
    plan_o = _oracle_plan(w.rules)
    Lo, Ro = api.CTable(w.left.cols), api.CTable(w.right.cols)
    filt = _stratified(Lo, plan_o, w.n_partitions, 32, 5)
    o = api.run_block(Lo, Ro, plan_o, w.n_partitions, left_row_filter=filt)
    mine = _rows_of(got, filt)
    assert len(o.pairs) > 1000
    assert np.array_equal(mine, o.pairs)
    assert o.fma_ambiguous == 0 and o.fp64_flips == 0


def test_c3_reduced_every_rule_alone(built, ctx, c3_small):
    """Each of the 8 rules alone (partitioned, as the reference does, on its
    own first equality) matches pairs of its own, and its sampled pairs equal
    the oracle's: the rule set is covered rule by rule."""
    w = c3_small
    L = hb.Table.from_columns(w.left.cols, ctx)
    R = hb.Table.from_columns(w.right.cols, ctx)
    Lo, Ro = api.CTable(w.left.cols), api.CTable(w.right.cols)
    for k, doc in enumerate(w.rules):
        plan = hb.Plan.from_yaml([doc], ctx)
        plan_o = _oracle_plan([doc])
        got, st = hb.block(ctx, plan, L, R, w.n_partitions, hb.INT_MAX, "batched")
        assert st.n_matches > 0, k
        filt = _stratified(Lo, plan_o, w.n_partitions, 16, 9 + k)
        o = api.run_block(Lo, Ro, plan_o, w.n_partitions, left_row_filter=filt)
        assert np.array_equal(_rows_of(got, filt), o.pairs), k


def test_c5_shape_sampled_parity(built, ctx):
    """The C5 shape (titles and authors of 64-256 characters, a Zipf key over
    2^20 values, 3 rules, 64 partitions) at 40k x 40k: one-shot and streamed
    windows give the same pairs, and a sample equals the oracle's."""
    w = synth_big.c5(40_000, 40_000, 800)
    plan = hb.Plan.from_yaml(w.rules, ctx)
    L = hb.Table.from_columns(w.left.cols, ctx)
    R = hb.Table.from_columns(w.right.cols, ctx)
    one, s1 = hb.block(ctx, plan, L, R, w.n_partitions, hb.INT_MAX, "batched")
    win, s2 = hb.block_streamed(ctx, plan, L, R, w.n_partitions, 24 << 20)
    assert s2.n_windows > 1
    assert np.array_equal(sorted_pairs(one), sorted_pairs(win))
    plan_o = _oracle_plan(w.rules)
    Lo, Ro = api.CTable(w.left.cols), api.CTable(w.right.cols)
    filt = _stratified(Lo, plan_o, w.n_partitions, 24, 3)
    o = api.run_block(Lo, Ro, plan_o, w.n_partitions, left_row_filter=filt)
    assert len(o.pairs) > 0
    assert np.array_equal(_rows_of(one, filt), o.pairs)


def test_serving_small_requests_against_1m_resident(built, ctx):
    """Requests of 3-20 records, submitted together, against a 1M-row
    resident table: each request's pairs equal the oracle's over the whole
    table."""
    right = synth_big.c4_right(1_000_000)
    reqs = synth_big.c4_requests(right, 6, sizes=[3, 7, 20, 12, 5, 16], seed=3, p_true=0.5)
    plans = [hb.Plan.from_yaml([d], ctx) for d in synth_big.SERVE_RULES]
    R = hb.Table.from_columns(right.cols, ctx)
    Ro = api.CTable(right.cols)
    with hb.Server(ctx, plans, R) as srv:
        for i, q in enumerate(reqs):
            srv.submit(i, q.rule, q.cols)
        got = {}
        while len(got) < len(reqs):
            r = srv.poll(-1)
            got[r["id"]] = r
    for i, q in enumerate(reqs):
        o = api.run_block(api.CTable(q.cols), Ro, _oracle_plan([synth_big.SERVE_RULES[q.rule]]), 1)
        assert got[i]["status"] == hb.OK
        assert np.array_equal(sorted_pairs(got[i]["pairs"]), o.pairs), i
