"""The partition hash restated in hyperblocker_gb300/csrc/std_hash.h equals the
host's own std::hash<std::string> (the reference's bucket function,
data_mngr.h:157, 187) on random byte strings of every length 0..300.

A small C++ program is compiled with the host compiler and compares both
functions; the device ingest uses the same header, and its buckets are
checked against the oracle (which calls std::hash) in test_gpu_ingest.py.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHECK = r"""
#include <cstdio>
#include <functional>
#include <random>
#include <string>
#include "std_hash.h"
int main() {
  std::mt19937_64 g(20261203);
  long bad = 0, n = 0;
  for (int len = 0; len <= 300; len++)
    for (int t = 0; t < 200; t++) {
      std::string s(len, '\0');
      for (auto& c : s) c = (char)(g() & 0xff);
      if (std::hash<std::string>{}(s) != hbx::std_hash_bytes((const uint8_t*)s.data(), s.size())) bad++;
      n++;
    }
  std::printf("%ld %ld\n", bad, n);
  return bad != 0;
}
"""


def test_std_hash_restatement_matches_std_hash(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "check.cpp"
    src.write_text(CHECK)
    exe = tmp_path / "check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "hyperblocker_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    bad, n = map(int, out.stdout.split())
    assert n == 301 * 200
    assert bad == 0 and out.returncode == 0
