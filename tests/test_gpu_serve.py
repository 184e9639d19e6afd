"""The serving loop (hbx_serve_*): resident right table, continuous batching.

Every request's pairs are compared with the oracle run on (the request's
records, the resident table) with the request's plan, one partition; the
same requests submitted one at a time and all at once (so that they share
batches) must give identical results.
"""
import time

import numpy as np
import pytest

import hyperblocker_gb300 as hb
from hyperblocker_gb300 import synth, synth_big
from oracle import api, rules
from tests import _util

pytestmark = pytest.mark.gpu


def _oracle_plan(docs):
    return rules.serialize(rules.sort_rules([rules.decode_rule(rules.parse_yaml(d)) for d in docs]))


def _cells(cols):
    return [[b[o[r]:o[r + 1]].tobytes() for r in range(len(o) - 1)] for b, o in cols]


@pytest.fixture(scope="module")
def resident(built):
    right = synth_big.c4_right(30000)
    reqs = synth_big.c4_requests(right, 24, rate=1e6, min_rows=1, max_rows=400, seed=3,
                                 p_true=0.2)
    return right, reqs


def _drain(srv, n, timeout_s=120.0):
    out, t0 = {}, time.time()
    while len(out) < n:
        r = srv.poll(1000)
        assert time.time() - t0 < timeout_s, "serving results did not arrive"
        if r is not None:
            out[r["id"]] = r
    return out


def _server(ctx, right, plan_docs, **kw):
    plans = [hb.Plan.from_yaml(d if isinstance(d, list) else [d], ctx) for d in plan_docs]
    R = hb.Table.from_columns(right.cols, ctx)
    return hb.Server(ctx, plans, R, **kw), R


def test_requests_match_the_oracle(ctx, resident):
    right, reqs = resident
    srv, _ = _server(ctx, right, synth_big.SERVE_RULES)
    for i, q in enumerate(reqs):
        srv.submit(i, q.rule, q.cols)
    got = _drain(srv, len(reqs))
    srv.close()
    R = api.CTable(right.to_columns())
    n_matches = 0
    for i, q in enumerate(reqs):
        r = got[i]
        assert r["status"] == hb.OK
        want = api.run_block(api.CTable(_cells(q.cols)), R,
                             _oracle_plan([synth_big.SERVE_RULES[q.rule]]), 1)
        assert np.array_equal(r["pairs"], want.pairs), i
        assert r["comparisons"] == want.pair_comparisons, i
        n_matches += len(want.pairs)
    assert n_matches > 0


def test_alone_and_in_the_mix_are_identical(ctx, resident):
    right, reqs = resident
    srv, _ = _server(ctx, right, synth_big.SERVE_RULES, max_inflight=2)
    alone = {}
    for i, q in enumerate(reqs):
        srv.submit(i, q.rule, q.cols)
        alone.update(_drain(srv, 1))
    for i, q in enumerate(reqs):
        srv.submit(100 + i, q.rule, q.cols)
    mixed = _drain(srv, len(reqs))
    st = srv.stats()
    srv.close()
    assert max(r["batch_requests"] for r in mixed.values()) > 1, "nothing was batched"
    for i in range(len(reqs)):
        assert alone[i]["batch_requests"] == 1
        assert np.array_equal(alone[i]["pairs"], mixed[100 + i]["pairs"]), i
        assert alone[i]["comparisons"] == mixed[100 + i]["comparisons"], i
    assert st.requests_done == 2 * len(reqs)


def test_multi_rule_plan_and_unseen_values(ctx, resident):
    right, reqs = resident
    docs = [synth.rule_yaml([4], [(1, 0.8)]), synth.rule_yaml([3, 4], [(2, 0.7)])]
    srv, _ = _server(ctx, right, [docs])
    # records with bytes and equality values the resident table never has
    q = reqs[5]
    cells = _cells(q.cols)
    n = len(cells[0])
    for r in range(0, n, 3):
        cells[1][r] = cells[1][r] + "#é~".encode()
        cells[3][r] = b"Nowhere Venue"
    for r in range(1, n, 5):
        cells[4][r] = b"1979"
    if n > 2:
        cells[1][2] = b"ab\x00cd"
    srv.submit(7, 0, cells)
    got = _drain(srv, 1)[7]
    srv.close()
    want = api.run_block(api.CTable(cells), api.CTable(right.to_columns()), _oracle_plan(docs), 1)
    assert np.array_equal(got["pairs"], want.pairs)


def test_budget_refuses_oversized_requests(ctx, resident):
    right, reqs = resident
    srv, _ = _server(ctx, right, synth_big.SERVE_RULES, budget_bytes=1 << 16)
    big = max(reqs, key=lambda q: q.n_rows)
    with pytest.raises(hb.HbxError) as e:
        srv.submit(1, big.rule, big.cols)
    assert e.value.status == hb.ERR_CAPACITY
    srv.close()


def test_empty_request(ctx, resident):
    right, _ = resident
    srv, _ = _server(ctx, right, synth_big.SERVE_RULES)
    srv.submit(3, 1, [[] for _ in range(5)])
    r = _drain(srv, 1)[3]
    srv.close()
    assert r["status"] == hb.OK and len(r["pairs"]) == 0
