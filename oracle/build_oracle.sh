#!/usr/bin/env bash
# Builds oracle/_build/liboracle.so (the CPU restatement, test infrastructure)
# and, when the reference tree is present, oracle/_ref/libquadprog_ref.so.
# Portable flags only: the same recipe runs on x86_64 and aarch64 hosts.
# -ffp-contract=off: no fused multiply-adds, so both hosts round every
# product and sum as written (the GPU ICA path reproduces that order).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
g++ -std=c++17 -O3 -ffp-contract=off -fopenmp -fPIC -shared -Wall -Wno-unused-function \
  "$HERE/oracle_capi.cpp" -o "$HERE/_build/liboracle.so"
echo "built $HERE/_build/liboracle.so"
bash "$HERE/build_ref.sh"  # skips when the reference tree is absent
