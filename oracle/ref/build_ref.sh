#!/usr/bin/env bash
# build_ref.sh -- TEST INFRASTRUCTURE ONLY.
#
# Compiles the reference's own kernel headers (core/gpu/global_func.cuh and
# core/gpu/device_func.cuh, read in place from the reference checkout) for the
# CPU with g++, together with oracle/ref/ref_driver.cpp, into
# oracle/_ref/libhb_ref.so.  Nothing from the reference is copied into this
# repository; the output directory is git-ignored.
#
# usage: oracle/ref/build_ref.sh REFERENCE_ROOT   (the reference checkout)
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
if [ $# -lt 1 ]; then
  echo "usage: build_ref.sh REFERENCE_ROOT" >&2
  exit 2
fi
ref="$1"
out="$here/../_ref"
if [ ! -f "$ref/core/gpu/global_func.cuh" ]; then
  echo "build_ref.sh: reference checkout not found at $ref" >&2
  exit 3
fi
mkdir -p "$out"
# -ffp-contract=off: the reference's host-side restatement must not fuse
# multiplies into adds on machines whose compilers do that by default.
g++ -std=c++17 -O2 -fPIC -shared -ffp-contract=off -w \
  -I "$here/shim_include" -I "$here" -I "$here/types_overlay" \
  -I "$ref" -I "$ref/core" \
  "$here/ref_driver.cpp" -o "$out/libhb_ref.so" -lpthread
echo "built $out/libhb_ref.so"
