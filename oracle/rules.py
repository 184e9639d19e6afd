"""Rule decoding and plan serialisation, restated -- TEST INFRASTRUCTURE ONLY.

Follows the reference:

* ``YAML::convert<Rule>::decode`` (core/common/yaml_config.h:37-75): only
  element ``[0]`` of Relations/Equalities/Sim/Threshold lists is read (plus
  Relations[1]); decoding happens only when ``Preconditions`` has exactly four
  keys; threshold ``k`` (list position ``2+k``) is keyed by the LEFT column of
  similarity predicate ``k`` (``sim[2 + 2k]``), first insertion wins;
  integers go through ``std::stoi`` and thresholds through ``std::stof``.
* ``ExecutionPlanGenerator`` (core/components/execution_plan_generator.h:64-155):
  rule files are read in directory order, sorted by the size of the
  equality vector (descending) with ``std::sort``, then each rule becomes
  its equality slots (threshold 1), its similarity slots (threshold of the
  slot's column) and one checkpoint slot (INT_MAX, ' ', 1).

yaml-cpp is an un-vendored submodule of the reference (.gitmodules:1-3, no
pinned version); this module parses only the YAML subset the rule format uses
(block mappings, block sequences of flow sequences, flow sequences, plain or
quoted scalars, comments), so YAML edge cases are parity-unpinned.
"""
from __future__ import annotations

import ctypes
import os
import math
import re
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

CHECK_POINT = 2147483647  # core/common/types.h:13 (INT_MAX)


class RuleError(ValueError):
    pass


# ----------------------------------------------------------------- YAML subset
def _strip_comment(line: str) -> str:
    out = []
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "\"'":
            q = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(ch)
    return "".join(out).rstrip()


def _scalar(tok: str) -> str:
    tok = tok.strip()
    if len(tok) >= 2 and tok[0] == tok[-1] and tok[0] in "\"'":
        return tok[1:-1]
    return tok


def _flow_seq(text: str) -> List[str]:
    text = text.strip()
    if not (text.startswith("[") and text.endswith("]")):
        raise RuleError(f"expected a flow sequence, got {text!r}")
    inner = text[1:-1].strip()
    if not inner:
        return []
    return [_scalar(t) for t in inner.split(",")]


def _value(text: str):
    text = text.strip()
    if text.startswith("["):
        return _flow_seq(text)
    return _scalar(text)


def parse_yaml(src: str):
    """Parse the block-structured subset into dicts / lists / strings."""
    lines = []
    for raw in src.splitlines():
        s = _strip_comment(raw.replace("\t", "  "))
        if s.strip() and s.strip() not in ("---", "..."):
            lines.append((len(s) - len(s.lstrip(" ")), s.strip()))
    pos = 0

    def block(indent):
        nonlocal pos
        if pos >= len(lines):
            return None
        ind, text = lines[pos]
        if not (text.startswith("- ") or text == "-") and not re.match(
                r"^([^:\[\]{}]+?)\s*:(?:\s+(.*))?$", text):
            # a plain or flow scalar on its own (more indented) line
            pos += 1
            return _value(text)
        if text.startswith("- ") or text == "-":
            seq = []
            while pos < len(lines) and lines[pos][0] == ind and (
                lines[pos][1].startswith("- ") or lines[pos][1] == "-"
            ):
                item = lines[pos][1][1:].strip()
                pos += 1
                if item:
                    seq.append(_value(item))
                else:
                    seq.append(block(lines[pos][0]) if pos < len(lines) and lines[pos][0] > ind else None)
            return seq
        mp: Dict[str, object] = {}
        while pos < len(lines) and lines[pos][0] == ind:
            text = lines[pos][1]
            m = re.match(r"^([^:\[\]{}]+?)\s*:(?:\s+(.*))?$", text)
            if not m:
                raise RuleError(f"cannot parse line {text!r}")
            key, rest = _scalar(m.group(1)), m.group(2)
            pos += 1
            if rest is not None and rest.strip():
                mp[key] = _value(rest)
            elif pos < len(lines) and lines[pos][0] > ind:
                mp[key] = block(lines[pos][0])
            elif pos < len(lines) and lines[pos][0] == ind and lines[pos][1].startswith("-"):
                mp[key] = block(ind)
            else:
                mp[key] = None
        return mp

    if not lines:
        return None
    out = block(lines[0][0])
    if pos != len(lines):
        raise RuleError(f"unparsed YAML from line {lines[pos][1]!r}")
    return out


# ----------------------------------------------------------------- decoding
def _stoi(s: str) -> int:
    """std::stoi: strtol base 10 after leading white space; out of int range
    throws."""
    m = re.match(r"^\s*([+-]?\d+)", s)
    if not m:
        raise RuleError(f"stoi: invalid argument {s!r}")
    v = int(m.group(1))
    if not -2**31 <= v <= 2**31 - 1:
        raise RuleError(f"stoi: out of range {s!r}")
    return v


def _stof(s: str) -> float:
    """std::stof: strtof's longest valid prefix -- decimal, hexadecimal
    (0x...p...), inf/infinity or nan/nan(...), case-insensitive, after
    leading white space -- rounded to float."""
    import numpy as np

    m = re.match(r"^\s*([+-]?)(0[xX](?:[0-9a-fA-F]+\.?[0-9a-fA-F]*|\.[0-9a-fA-F]+)(?:[pP][+-]?\d+)?"
                 r"|(?i:infinity|inf|nan(?:\([0-9A-Za-z_]*\))?)"
                 r"|\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?)", s)
    if not m:
        raise RuleError(f"stof: invalid argument {s!r}")
    sign, body = m.group(1), m.group(2)
    numeric = body[0].isdigit() or body[0] == "."
    if body[:2] in ("0x", "0X"):
        v = float.fromhex(body if "p" in body.lower() else body + "p0")
    elif numeric:
        v = float(body)
    else:
        v = float(body.split("(")[0])
    v = -v if sign == "-" else v
    if numeric:  # strtof sets ERANGE (std::stof throws) when a number over- or underflows
        with np.errstate(over="ignore"):  # the float32 overflow is the check
            f = abs(float(np.float32(v))) if np.isfinite(v) else math.inf
        if math.isinf(f) or (v != 0.0 and f < float(np.finfo(np.float32).tiny)):
            raise RuleError(f"stof: out of range {s!r}")
    return float(np.float32(v))


def _strlist(node) -> List[str]:
    if isinstance(node, list):
        return [x if isinstance(x, str) else str(x) for x in node]
    if isinstance(node, str):
        return [node]
    raise RuleError("expected a sequence")


def _idx(node, i):
    if not isinstance(node, list) or i >= len(node):
        raise RuleError("missing sequence element")
    return node[i]


@dataclass
class Rule:
    relation_l: List[int] = field(default_factory=list)
    relation_r: List[int] = field(default_factory=list)
    eq: List[int] = field(default_factory=list)
    sim: List[int] = field(default_factory=list)
    threshold: Dict[int, float] = field(default_factory=dict)
    con_eq: List[int] = field(default_factory=list)


def decode_rule(doc) -> Rule:
    """yaml_config.h:37-75."""
    if not isinstance(doc, dict) or len(doc) < 2:
        raise RuleError("Invalid rule's metadata format")
    pre = doc.get("Preconditions")
    if not isinstance(pre, dict):
        raise RuleError("missing Preconditions")
    rel = pre.get("Relations")
    relation_l = _strlist(_idx(rel, 0))
    relation_r = _strlist(_idx(rel, 1))
    r = Rule()
    if len(pre) == 4:
        r.relation_l = [_stoi(x) for x in relation_l]
        r.relation_r = [_stoi(x) for x in relation_r]
        r.eq = [_stoi(x) for x in _strlist(_idx(pre.get("Equalities"), 0))]
        r.sim = [_stoi(x) for x in _strlist(_idx(pre.get("Sim"), 0))]
        thr = _strlist(_idx(pre.get("Threshold"), 0))
        for i in range(2, len(thr)):
            k = 2 + (i - 2) * 2
            if k >= len(r.sim):
                raise RuleError("threshold without a similarity predicate")
            r.threshold.setdefault(r.sim[k], _stof(thr[i]))
        con = doc.get("Conseq")
        if isinstance(con, dict) and con.get("Equality") is not None:
            r.con_eq = [_stoi(x) for x in _strlist(con.get("Equality"))]
    return r


def validate_rule(r: Rule, where: str = "") -> None:
    """Rules the reference cannot run (undefined behaviour there) are refused."""
    if len(r.eq) < 2 or len(r.sim) < 2:
        raise RuleError(f"{where}: rule was not decoded (Preconditions must have 4 keys)")
    if (len(r.eq) - 2) % 2 or (len(r.sim) - 2) % 2:
        raise RuleError(f"{where}: predicate lists must hold column pairs")
    if len(r.eq) == 2 and len(r.sim) == 2:
        raise RuleError(f"{where}: rule has no predicate")
    for k in range(2, len(r.sim), 2):
        if r.sim[k] not in r.threshold:
            raise RuleError(f"{where}: similarity predicate on column {r.sim[k]} has no threshold")


def load_rule_dir(rule_dir: str) -> Tuple[List[str], List[Rule]]:
    """Rule files in directory (readdir) order, like directory_iterator."""
    names = [e.name for e in os.scandir(rule_dir)]
    rules = []
    for n in names:
        p = os.path.join(rule_dir, n)
        with open(p, "r") as f:
            r = decode_rule(parse_yaml(f.read()))
        validate_rule(r, p)
        rules.append(r)
    return names, rules


def sort_rules(rules: List[Rule], lib: Optional[ctypes.CDLL] = None) -> List[Rule]:
    """execution_plan_generator.h:75-79, via libstdc++'s std::sort itself."""
    if lib is None:
        from . import api

        lib = api.lib()
    n = len(rules)
    sizes = (ctypes.c_int32 * max(n, 1))(*[len(r.eq) for r in rules])
    perm = (ctypes.c_int32 * max(n, 1))()
    lib.hbo_sort_rules(sizes, n, perm)
    return [rules[perm[i]] for i in range(n)]


@dataclass
class Plan:
    pred_index: List[int]
    pred_type: bytes
    pred_threshold: List[float]

    @property
    def length(self) -> int:
        return len(self.pred_index)


def serialize(rules_sorted: List[Rule]) -> Plan:
    """execution_plan_generator.h:111-137 (kEqualitiesFirst)."""
    pi: List[int] = []
    pt = bytearray()
    th: List[float] = []
    for r in rules_sorted:
        for x in r.eq[2:]:
            pi.append(x)
            pt += b"e"
            th.append(1.0)
        for x in r.sim[2:]:
            pi.append(x)
            pt += b"s"
            # the right slot's threshold is never read by the kernel
            th.append(r.threshold.get(x, 1.0))
        pi.append(CHECK_POINT)
        pt += b" "
        th.append(1.0)
    return Plan(pi, bytes(pt), th)


def plan_from_dir(rule_dir: str) -> Plan:
    _, rules = load_rule_dir(rule_dir)
    return serialize(sort_rules(rules))
