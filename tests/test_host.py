"""Host logic of the engine without a GPU: CSV tokenization, YAML rule
decoding, plan serialization and ordering, error statuses, output writer."""
import os

import numpy as np
import pytest

import hyperblocker_gb300 as hb
from oracle import api, csvref, rules
from hyperblocker_gb300 import synth

README_RULE = """Preconditions:
  # There are two relation tables, each with 5 columns.
  Relations:
    - [0, 0, 1, 2, 3, 4]
    - [1, 0, 1, 2, 3, 4]
  # The equality predicate is on the 4th column.
  Equalities:
    - [0, 1, 4, 4]
  Sim:
    - [0, 1, 1, 1, 2, 2]
  Threshold:
    - [0, 1, 0.89, 0.85]
Conseq:
  Option:
    Equality
  # The ID is in the 0th column.
  Equality:
    [0, 1, 0, 0]
"""


@pytest.mark.parametrize("data", [
    b'"id","t"\r\n1,"a, b"\r\n2,"say ""hi"""\r\n',
    b'id,t\n1,plain\n2,"quoted"\n3,',
    b'\xef\xbb\xbfid,t\n1,x\n',
    b'a,b\n"x""y",z\n"q",w"x\n',
    b'a,b\n1,\n,2\n',
])
def test_csv_matches_rapidcsv_restatement(built, tmp_path, data):
    p = tmp_path / "t.csv"
    p.write_bytes(data)
    want = csvref.read_columns(str(p))
    t = hb.Table.from_csv(str(p))
    assert t.n_rows == len(want[0])
    assert t.n_cols == len(want)
    # ids come back through the writer, byte for byte
    out = tmp_path / "o.csv"
    n = t.n_rows
    pairs = np.stack([np.arange(n), np.arange(n)], 1).astype(np.uint32)
    hb.write_pairs(t, t, pairs, str(out))
    got = out.read_bytes().split(b"\n")[:-1]
    assert got == [c.split(b"\0")[0] + b"," + c.split(b"\0")[0] for c in want[0]]


@pytest.mark.parametrize("data", [b"a,b,c\n1,2\n", b'a,b\n"unterminated,q\n'])
def test_csv_short_row_is_parse_error(built, tmp_path, data):
    """rapidcsv's GetColumn throws on a short row; the engine reports PARSE."""
    p = tmp_path / "t.csv"
    p.write_bytes(data)
    with pytest.raises(ValueError):
        csvref.read_columns(str(p))
    with pytest.raises(hb.HbxError) as e:
        hb.Table.from_csv(str(p))
    assert e.value.status == hb.ERR_PARSE


def _oracle_plan(docs):
    api.build()
    return rules.serialize(rules.sort_rules([rules.decode_rule(rules.parse_yaml(d)) for d in docs]))


@pytest.mark.parametrize("docs", [
    [README_RULE],
    [synth.rule_yaml([4], [(1, 0.89), (2, 0.85)]), synth.rule_yaml([3], [(1, 0.95)])],
    [synth.rule_yaml([], [(1, 0.7)]), synth.rule_yaml([3, 4], [(2, 0.8)]),
     synth.rule_yaml([4], [(1, 0.6)])],
    # 20 rules: std::sort is not an insertion sort above 16 elements
    [synth.rule_yaml([3] * (k % 3), [(1, 0.5 + 0.01 * k)]) for k in range(20)],
    # two similarities on the same left column: the first threshold wins
    [README_RULE.replace("[0, 1, 1, 1, 2, 2]", "[0, 1, 1, 1, 1, 2]")],
    # thresholds std::stof reads besides decimals: nan, infinities, hexadecimal
    [README_RULE.replace("[0, 1, 0.89, 0.85]", "[0, 1, nan, -inf]"),
     README_RULE.replace("[0, 1, 0.89, 0.85]", "[0, 1, inf, 0x1.8p-1]")],
])
def test_plan_matches_reference_serialization(built, docs):
    want = _oracle_plan(docs)
    p = hb.Plan.from_yaml(docs)
    pi, pt, th = p.serialized()
    assert pi == want.pred_index
    assert pt == want.pred_type
    assert np.array_equal(np.float32(th), np.float32(want.pred_threshold), equal_nan=True)
    assert p.n_rules == len(docs)


@pytest.mark.parametrize("doc,status", [
    ("Preconditions:\n  Relations:\n    - [0]\n    - [1]\n  Equalities:\n    - [0, 1, 4, 4]\n"
     "  Sim:\n    - [0, 1, 1, 1]\nConseq:\n  Equality:\n    [0, 1, 0, 0]\n", hb.ERR_UNSUPPORTED),
    ("just: one\n", hb.ERR_PARSE),
    ("Preconditions:\n  Relations: [\n", hb.ERR_PARSE),
    (README_RULE.replace("[0, 1, 0.89, 0.85]", "[0, 1, 0.89]"), hb.ERR_UNSUPPORTED),
    (README_RULE.replace("[0, 1, 4, 4]", "[0, 1, 4]"), hb.ERR_UNSUPPORTED),
    (README_RULE.replace("[0, 1, 4, 4]", "[0, 1, x, 4]"), hb.ERR_PARSE),
])
def test_bad_rules_are_refused(built, doc, status):
    with pytest.raises(hb.HbxError) as e:
        hb.Plan.from_yaml([doc])
    assert e.value.status == status


def test_rule_dir_errors(built, tmp_path):
    with pytest.raises(hb.HbxError) as e:
        hb.Plan.from_rule_dir(str(tmp_path / "missing"))
    assert e.value.status == hb.ERR_IO
    (tmp_path / "r").mkdir()
    with pytest.raises(hb.HbxError) as e:
        hb.Plan.from_rule_dir(str(tmp_path / "r"))
    assert e.value.status == hb.ERR_PARSE


def test_rule_dir_order_is_directory_order(built, tmp_path):
    d = tmp_path / "rules"
    d.mkdir()
    docs = [synth.rule_yaml([4], [(1, 0.89)]), synth.rule_yaml([3], [(1, 0.95)])]
    for k, doc in enumerate(docs):
        (d / f"{k}.yaml").write_text(doc)
    want = rules.plan_from_dir(str(d))
    pi, pt, th = hb.Plan.from_rule_dir(str(d)).serialized()
    assert pi == want.pred_index and pt == want.pred_type


def test_cli_rejects_unknown_flag(built):
    assert hb.run_cli(["run_hyperblocker_exec", "-no_such_flag=1"]) == 1
    assert hb.run_cli(["run_hyperblocker_exec", "-n_partitions=abc"]) == 1
    assert hb.run_cli(["run_hyperblocker_exec", "-hbx_mode=fast"]) == 1


@pytest.mark.parametrize("argv", [
    ["-data_l"],                               # string flag without its argument
    ["-n_partitions"],                         # number flag without its argument
    ["-n_partitions", "-1x"],
    ["-read_header=maybe"],
    ["-prefix_hash_pred_idx=3000000000"],      # above INT_MAX
    ["-hbx_device=gpu0"],
    ["stray_argument"],
])
def test_cli_flag_errors(built, argv):
    """Malformed command lines end with exit code 1 before any device work."""
    assert hb.run_cli(["run_hyperblocker_exec"] + argv) == 1


@pytest.mark.parametrize("argv", [
    ["-rule_dir", "/nonexistent/rules", "-n_partitions", "8", "-sep", ";"],
    ["--rule_dir=/nonexistent/rules", "--n_partitions=0x10", "-read_header", "-scheduler=RR"],
    ["-rule_dir=/nonexistent/rules", "-noread_header", "-prefix_hash_pred_idx", "2",
     "-hbx_mode", "plain"],
])
def test_cli_accepts_gflags_forms(built, argv):
    """-flag=value, --flag=value, -flag value, bare booleans and -noflag all
    parse (gflags syntax, examples/run_hyperblocker.cu:22-31); the run then
    stops at the missing rule directory (or at the context where there is
    no GPU) with exit code 2, not at the flags."""
    assert hb.run_cli(["run_hyperblocker_exec"] + argv) == 2


def test_host_writer_lines(built, tmp_path):
    """hbx_write_pairs without a context (the host loop) appends one
    `id_l,id_r` line per pair, each id printed as a C string -- up to its
    first NUL -- like WriteMatch (core/components/host_reducer.h:80-90);
    commas and quotes inside ids are written as they are; a row index past
    the table is refused."""
    ids_l = [b"id", b"a1", b"x\x00hidden", b'"q,1"', b""]
    ids_r = [b"id", b"r0", b"r,1", b"\x00", b"long" * 40]
    L = hb.Table.from_columns([ids_l, [b"c"] * len(ids_l)])
    R = hb.Table.from_columns([ids_r, [b"c"] * len(ids_r)])
    pairs = np.array([[1, 1], [2, 2], [3, 3], [4, 4], [0, 0], [1, 4]], dtype=np.uint32)
    out = tmp_path / "pairs.csv"
    hb.write_pairs(L, R, pairs, str(out))
    cut = lambda b: b.split(b"\x00", 1)[0]
    want = b"".join(cut(ids_l[a]) + b"," + cut(ids_r[b]) + b"\n" for a, b in pairs)
    assert out.read_bytes() == want
    hb.write_pairs(L, R, pairs[:2], str(out))  # append mode
    assert out.read_bytes() == want + want[:want.index(b"\n", want.index(b"\n") + 1) + 1]
    with pytest.raises(hb.HbxError) as e:
        hb.write_pairs(L, R, np.array([[5, 0]], dtype=np.uint32), str(tmp_path / "bad.csv"))
    assert e.value.status == hb.ERR_INVALID_ARG


def test_column_ingest_refuses_bad_offsets(built):
    """hbx_table_ingest checks the caller's offsets: decreasing offsets are
    HBX_ERR_INVALID_ARG; offsets that do not start at 0 are taken relative to
    their first entry; columns of different lengths never reach the C ABI."""
    blob = np.frombuffer(b"abcdef", dtype=np.uint8)
    with pytest.raises(hb.HbxError) as e:
        hb.Table.from_columns([(blob, np.array([0, 3, 2, 6], dtype=np.int64))])
    assert e.value.status == hb.ERR_INVALID_ARG
    t = hb.Table.from_columns([(blob, np.array([2, 3, 6], dtype=np.int64))])
    b, o = t.column(0)
    assert bytes(b) == b"cdef" and list(o) == [0, 1, 4]
    with pytest.raises(ValueError):
        hb.Table.from_columns([[b"a", b"b"], [b"c"]])



@pytest.mark.parametrize("col,status", [("2147483648", hb.ERR_PARSE), ("99999999999", hb.ERR_PARSE),
                                        ("-2147483649", hb.ERR_PARSE)])
def test_out_of_range_column_index_is_refused_like_stoi(built, col, status):
    """std::stoi throws out_of_range beyond int (yaml_config.h reads column
    indices with it): the engine refuses the rule, and the oracle's
    restatement raises."""
    from oracle import rules

    doc = README_RULE.replace("[0, 1, 4, 4]", f"[0, 1, {col}, 4]")
    with pytest.raises(hb.HbxError) as e:
        hb.Plan.from_yaml([doc])
    assert e.value.status == status
    with pytest.raises(rules.RuleError):
        rules.decode_rule(rules.parse_yaml(doc))
