"""libhbx.so loads and exports every function include/hbx.h declares, and a
plain C program built against the header drives its host-side calls (no GPU)."""
import os
import re
import shutil
import subprocess

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


C_CLIENT = r"""
#include <stdio.h>
#include <string.h>
#include "hbx.h"

int main(int argc, char** argv) {
  if (argc != 3) return 90;
  hbx_plan* plan = NULL;
  if (hbx_plan_from_rule_dir(NULL, argv[1], &plan) != HBX_OK) return 91;
  const char* cells_l = "idl1l2";
  const int64_t off_l[4] = {0, 2, 4, 6};
  const char* cells_r = "idr1";
  const int64_t off_r[3] = {0, 2, 4};
  const char* data_l[2] = {cells_l, cells_l};
  const int64_t* offs_l[2] = {off_l, off_l};
  const char* data_r[2] = {cells_r, cells_r};
  const int64_t* offs_r[2] = {off_r, off_r};
  hbx_columns cl = {3, 2, data_l, offs_l};
  hbx_columns cr = {2, 2, data_r, offs_r};
  hbx_table *L = NULL, *R = NULL;
  if (hbx_table_ingest(NULL, &cl, &L) != HBX_OK || hbx_table_ingest(NULL, &cr, &R) != HBX_OK)
    return 92;
  const uint32_t l_row[2] = {1, 2}, r_row[2] = {1, 1};
  if (hbx_write_pairs(NULL, L, R, l_row, r_row, 2, argv[2]) != HBX_OK) return 93;
  const uint32_t bad[1] = {7};
  hbx_status s = hbx_write_pairs(NULL, L, R, bad, r_row, 1, argv[2]);
  printf("%d %lld %s|%s\n", hbx_plan_n_rules(plan), (long long)hbx_table_n_rows(L),
         hbx_status_string(s), hbx_last_error(NULL));
  hbx_table_destroy(L);
  hbx_table_destroy(R);
  hbx_plan_destroy(plan);
  return 0;
}
"""


def test_plain_c_client(built, tmp_path):
    """The header is C99; a C program links libhbx.so and runs the host-side
    calls a cgo or ctypes binding would make first: a plan from a rule
    directory, tables from caller cells, id lines appended to a file, and a
    refused row index reported through the status and the last error."""
    gcc = shutil.which("gcc")
    if gcc is None:
        import pytest

        pytest.skip("no C compiler")
    from hyperblocker_gb300 import synth

    src = tmp_path / "client.c"
    src.write_text(C_CLIENT)
    exe = tmp_path / "client"
    lib_dir = os.path.dirname(hb.LIB_PATH)
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), "-L", lib_dir, "-lhbx", "-Wl,-rpath," + lib_dir, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rules = tmp_path / "rules"
    rules.mkdir()
    (rules / "0.yaml").write_text(synth.rule_yaml([1], [(1, 0.9)]))
    out = tmp_path / "pairs.csv"
    r = subprocess.run([str(exe), str(rules), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
    n_rules, n_rows, rest = r.stdout.strip().split(" ", 2)
    assert (n_rules, n_rows) == ("1", "3")
    assert rest.startswith("invalid argument|") and "out of range" in rest
    assert out.read_bytes() == b"l1,r1\nl2,r1\n"

