"""libhbx.so loads and exports every function include/hbx.h declares (no GPU)."""
import os
import re

import hyperblocker_gb300 as hb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "hbx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(hbx_[a-z_]+)\s*\(", src)
    return sorted(set(n for n in names))


def test_every_declared_symbol_is_exported(built):
    L = hb.lib()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
        assert n in hb.SIGNATURES, f"{n} has no ctypes signature"


def test_status_strings(built):
    L = hb.lib()
    for s in range(10):
        assert L.hbx_status_string(s) != b"unknown status"
