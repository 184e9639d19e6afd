"""Generates tests/golden/*.json from the reference's own kernel.

Run here, where the reference checkout exists (it does not on GPU machines):

    python tests/golden/make_golden.py [REFERENCE_ROOT]

For every case the candidate pairs come from the reference's
``blocking_kernel`` compiled for the CPU (``oracle/_ref/libhb_ref.so``), and the
C++ oracle port must agree pair for pair before anything is written.  A
fixture holds the match count and the SHA-256 of the sorted ``id_l,id_r\\n``
lines (the reference's output format), plus, for small cases, the pairs.

Cases
-----
* ``dblp_acm``: the reference's shipped DBLP-ACM tables and rule, with the
  thresholds 0.89/0.85 and the shipped 0.81/0.79 (known answers 1995 and 2477
  pairs).  Only counts and digests are stored; the tables stay in the
  reference checkout.
* ``synthetic``: seeded tables from hyperblocker_gb300.synth (C1 and C2
  shapes), for both directory orders of C2's two equal-rank rules, plus small
  edge cases (empty strings, long strings above 256 bytes, several
  partitions, the prefix hash).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import api, csvref, rules  # noqa: E402
from hyperblocker_gb300 import synth  # noqa: E402


def digest(lines):
    h = hashlib.sha256()
    for a, b in lines:
        h.update(a + b"," + b + b"\n")
    return h.hexdigest()


def ref_and_port(cols_l, cols_r, plan, n_part, prefix=2147483647):
    L, R = api.CTable(cols_l), api.CTable(cols_r)
    ref = api.run_ref_block(L, R, plan, n_part, prefix)
    port = api.run_block(L, R, plan, n_part, prefix)
    mine = sorted((cols_l[0][l], cols_r[0][r]) for l, r in port.pairs)
    if mine != ref:
        raise SystemExit("oracle port and reference kernel disagree")
    return ref, port


def plan_of(docs):
    rs = [rules.decode_rule(rules.parse_yaml(d)) for d in docs]
    return rules.serialize(rules.sort_rules(rs))


def edge_tables():
    """Small hand-made tables covering the edge cases the path has."""
    long_a = ("Ab, " * 80)[:300]
    long_b = ("Ab, " * 79 + "Ac, ")[:296]
    left = [
        [b"id", b"1", b"2", b"3", b"4", b"5", b"6", b"7", b"8"],
        [b"title", b"", b"", b"abc", b"martha", b"dwayne", b"dixon", long_a.encode(), b"x" * 70],
        [b"authors", b"a", b"", b"b", b"c", b"d", b"e", long_b.encode(), b"y" * 65],
        [b"venue", b"v1", b"v2", b"v1", b"v1", b"v2", b"v3", b"v1", b"v1"],
        [b"year", b"2000", b"2000", b"2001", b"2000", b"2000", b"2001", b"2000", b"2000"],
    ]
    right = [
        [b"id", b"a", b"b", b"c", b"d", b"e", b"f", b"g", b"h", b"i"],
        [b"title", b"", b"abd", b"marhta", b"duane", b"dicksonx", long_b.encode(), b"x" * 69 + b"z",
         b"abc", b"y"],
        [b"authors", b"", b"b", b"c", b"dd", b"e", long_a.encode(), b"y" * 64, b"q", b"a"],
        [b"venue", b"v1", b"v1", b"v1", b"v2", b"v3", b"v1", b"v1", b"v2", b"v2"],
        [b"year", b"2000", b"2001", b"2000", b"2000", b"2001", b"2000", b"2000", b"2001", b"2000"],
    ]
    return left, right


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else api.REFERENCE_ROOT
    api.REFERENCE_ROOT = ref_root
    api.build(force=True)
    if not api.ref_available():
        raise SystemExit("the reference kernel could not be built")
    out = {"generator": "tests/golden/make_golden.py", "cases": {}}

    # ---- DBLP-ACM known answers
    d = os.path.join(ref_root, "data", "dblp-acm")
    if os.path.isdir(d):
        A = csvref.read_columns(os.path.join(d, "tableA.csv"))
        B = csvref.read_columns(os.path.join(d, "tableB.csv"))
        M = csvref.read_columns(os.path.join(d, "match.csv"))
        truth = set(zip(M[0], M[1]))
        src = open(os.path.join(d, "rules", "0.yaml")).read()
        for thr in ("0.89, 0.85", "0.81, 0.79"):
            plan = plan_of([src.replace("0.81, 0.79", thr)])
            ref, port = ref_and_port(A, B, plan, 1)
            out["cases"][f"dblp_acm_{thr.replace(', ', '_')}"] = {
                "kind": "dblp_acm", "thresholds": thr, "n_partitions": 1,
                "count": len(ref), "true_positives": len(set(ref) & truth),
                "sha256": digest(ref), "pair_comparisons": port.pair_comparisons,
                "pairs_covered": port.pairs_covered}
            print("dblp_acm", thr, len(ref))

    # ---- synthetic workloads
    for name in ("c1", "c2"):
        w = synth.WORKLOADS[name]()
        cl, cr = synth.table_bytes(w.tables.left), synth.table_bytes(w.tables.right)
        orders = [list(range(len(w.rules)))]
        if len(w.rules) == 2:
            orders.append([1, 0])
        for order in orders:
            docs = [w.rules[k] for k in order]
            plan = plan_of(docs)
            ref, port = ref_and_port(cl, cr, plan, w.n_partitions)
            key = f"{name}_order_{''.join(map(str, order))}"
            out["cases"][key] = {
                "kind": "synthetic", "workload": name, "rule_order": order,
                "n_partitions": w.n_partitions, "count": len(ref), "sha256": digest(ref),
                "pair_comparisons": port.pair_comparisons, "pairs_covered": port.pairs_covered,
                "left_sha256": hashlib.sha256(b"\0".join(b"\1".join(c) for c in cl)).hexdigest(),
                "right_sha256": hashlib.sha256(b"\0".join(b"\1".join(c) for c in cr)).hexdigest()}
            print(key, len(ref))

    # ---- edge cases
    el, er = edge_tables()
    edge_rules = {
        "edge_title_authors": ([synth.rule_yaml([4], [(1, 0.8), (2, 0.7)])], 1, 2147483647),
        "edge_title_only_no_eq": ([synth.rule_yaml([], [(1, 0.75)])], 1, 2147483647),
        "edge_two_rules_3parts": ([synth.rule_yaml([4], [(1, 0.8)]),
                                   synth.rule_yaml([3, 4], [(2, 0.7), (1, 0.5)])], 3, 2147483647),
        "edge_prefix_hash": ([synth.rule_yaml([4], [(1, 0.5)])], 4, 1),
        "edge_eq_only": ([synth.rule_yaml([3, 4], [])], 2, 2147483647),
        "edge_threshold_one": ([synth.rule_yaml([], [(1, 1.0), (2, 0.0)])], 1, 2147483647),
    }
    for key, (docs, n_part, prefix) in edge_rules.items():
        plan = plan_of(docs)
        ref, port = ref_and_port(el, er, plan, n_part, prefix)
        out["cases"][key] = {
            "kind": "edge", "rules": docs, "n_partitions": n_part, "prefix_idx": prefix,
            "count": len(ref), "sha256": digest(ref),
            "pairs": [[a.decode(), b.decode()] for a, b in ref]}
        print(key, len(ref))

    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
