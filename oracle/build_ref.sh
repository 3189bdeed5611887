#!/usr/bin/env bash
# Builds oracle/_ref/libquadprog_ref.so from the reference's vendored
# QuadProg++ sources, compiled where they lie in the read-only reference tree
# (nothing is copied into this repository), plus oracle/quadprog_ref.cpp.
# The reference's MPRGP headers themselves cannot be built here: they need
# Eigen3 and Boost, which this image does not have.
# Usage: oracle/build_ref.sh [reference_root]
# The reference tree: the argument, else $MPRGP_REFERENCE_ROOT, else the
# build container's copy at /root/reference; without one it skips.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${MPRGP_REFERENCE_ROOT:-/root/reference}}"
QP="$REF/src/MPRGPSolver/SimpleQP"
if [ ! -f "$QP/QuadProg.cpp" ]; then
  echo "reference QuadProg++ sources not found under $QP; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++14 -O2 -fPIC -shared -w -I"$QP" \
  "$HERE/quadprog_ref.cpp" "$QP/QuadProg.cpp" "$QP/Array.cpp" \
  -o "$HERE/_ref/libquadprog_ref.so"
echo "built $HERE/_ref/libquadprog_ref.so"
