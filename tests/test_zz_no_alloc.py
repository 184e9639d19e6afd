"""hbx_block_static, the entry point for callers that cannot allocate device
memory (a host application whose device memory is handed out by another
runtime, a fixed device-memory budget, or a loop that cannot pay for
cudaMalloc's device synchronization).  It must give exactly the pairs the
ordinary hbx_block gives, call after call, although every call reuses the same
static scratch array inside the library.

This file is collected last on purpose, so that a run that stops at its first
failure has already run every other test.  It creates its own context and
runs alone in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

import hyperblocker_gb300 as hb
from hyperblocker_gb300 import synth
from tests import _util

pytestmark = pytest.mark.gpu


def _static_pairs(plan, L, R, n_part, capacity, free_bytes=None):
    """One hbx_block_static call into caller-owned device buffers.  With
    free_bytes (a list), the device's free memory just before and just after
    the call is appended to it: the call itself allocates nothing."""
    import torch

    out_l = torch.full((capacity,), -1, dtype=torch.int32, device="cuda")
    out_r = torch.full((capacity,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    p = hb.Pairs(out_l.data_ptr(), out_r.data_ptr(), capacity, 0, 0)
    st = hb.Stats()
    if free_bytes is not None:
        free_bytes.append(torch.cuda.mem_get_info()[0])
    status = hb.lib().hbx_block_static(0, plan.h, L.h, R.h, n_part, hb.INT_MAX, ctypes.byref(p),
                                       None, ctypes.byref(st))
    if free_bytes is not None:
        free_bytes.append(torch.cuda.mem_get_info()[0])
    if status != hb.OK:
        raise hb.HbxError(status, hb.lib().hbx_static_last_error().decode())
    n = int(p.n_written)
    pairs = np.stack([out_l[:n].cpu().numpy().view(np.uint32),
                      out_r[:n].cpu().numpy().view(np.uint32)], axis=1)
    return _util.sorted_pairs(pairs), st


def _oracle_pairs(cl, cr, docs, n_part):
    from oracle import api, rules

    plan = rules.serialize(rules.sort_rules([rules.decode_rule(rules.parse_yaml(d)) for d in docs]))
    return api.run_block(api.CTable(cl), api.CTable(cr), plan, n_part).pairs


@pytest.mark.parametrize("case", ["c1", "random_multi_rule"])
def test_static_scratch_matches_hbx_block_twice(case):
    ctx = hb.Context(0)
    if case == "c1":
        w = synth.c1()
        cl, cr = synth.table_bytes(w.tables.left), synth.table_bytes(w.tables.right)
        docs, n_part = w.rules, w.n_partitions
    else:
        cl, cr = _util.random_tables(7, 300, 900, b"abcdefgh ,", 100)
        docs = [synth.rule_yaml([3], [(1, 0.7)]), synth.rule_yaml([4], [(2, 0.6), (1, 0.5)])]
        n_part = 3
    plan = hb.Plan.from_yaml(docs, ctx)
    L = hb.Table.from_columns(cl, ctx)
    R = hb.Table.from_columns(cr, ctx)
    want, st_want = hb.block(ctx, plan, L, R, n_part, hb.INT_MAX, "batched")
    want = _util.sorted_pairs(want)
    assert len(want) > 0
    # the existing entry point is itself checked against the oracle
    assert np.array_equal(want, _oracle_pairs(cl, cr, docs, n_part))
    cap = len(want) + 1024
    free = []
    for k in range(2):  # two calls in a row share the static scratch
        got, st = _static_pairs(plan, L, R, n_part, cap, free if k == 1 else None)
        assert np.array_equal(got, want)
        assert st.pair_comparisons == st_want.pair_comparisons
        assert st.n_matches == len(want)
        assert 0 < st.h2d_bytes < 64 << 20  # bytes this call copied to the device
        assert st.ingest_on_device == 1  # encoded by the device encoder, inside the scratch
    # the second call (the array's address already looked up) allocates no
    # device memory
    assert free[0] == free[1]
    # too small an output: CAPACITY with the required count
    with pytest.raises(hb.HbxError) as e:
        _static_pairs(plan, L, R, n_part, max(1, len(want) // 2))
    assert e.value.status == hb.ERR_CAPACITY
    ctx.close()


def test_static_scratch_refuses_oversize_input():
    """An input beyond the 64 MiB scratch is refused with a clear error and no
    GPU work is started."""
    n = 300000
    left = [[b"id"] + [b"%d" % i for i in range(n)], [b"t"] + [b"x" * 200] * n]
    plan = hb.Plan.from_yaml([synth.rule_yaml([], [(1, 0.9)])])
    L = hb.Table.from_columns(left)
    p = hb.Pairs(0, 0, 0, 0, 0)
    status = hb.lib().hbx_block_static(0, plan.h, L.h, L.h, 1, hb.INT_MAX, ctypes.byref(p), None,
                                       None)
    assert status == hb.ERR_INVALID_ARG
    assert b"static scratch holds" in hb.lib().hbx_static_last_error()


def test_static_scratch_large_capacity_small_input():
    """A generous output buffer does not make a small multi-rule input
    overflow the scratch: the duplicate set is sized from what the
    partitions can hold, not from the capacity alone."""
    ctx = hb.Context(0)
    cl, cr = _util.random_tables(3, 50, 80, b"abcdef ,", 30)
    docs = [synth.rule_yaml([3], [(1, 0.6)]), synth.rule_yaml([4], [(2, 0.5)])]
    plan = hb.Plan.from_yaml(docs, ctx)
    L = hb.Table.from_columns(cl, ctx)
    R = hb.Table.from_columns(cr, ctx)
    got, st = _static_pairs(plan, L, R, 3, 16 << 20)
    assert np.array_equal(got, _oracle_pairs(cl, cr, docs, 3))
    ctx.close()
