#!/usr/bin/env bash
# ORACLE build recipe (test infrastructure only).
# Compiles the reference's own sources, unmodified and where they lie, into
# oracle/_ref/librr_ref.so, against the self-written Eigen subset in
# oracle/eigen_shim/ (the vendored Eigen lacks Eigen/Core).  Runs only where
# the reference checkout exists; the GPU host never builds or loads this.
#   usage: oracle/build_ref.sh [--if-present] [--stock] [REFERENCE_ROOT]
# The reference checkout is REFERENCE_ROOT, else $RILS_ROLS_REFERENCE, else
# /root/reference.  With --if-present a missing checkout is not an error
# (nothing is built).  --stock builds oracle/_ref/librr_ref_stock.so instead:
# the same sources with the C library's transcendentals, index-order sums and
# the reference's own flags (setup.py:14), for measuring how far the pinned
# arithmetic is from a stock build (eigen_shim/stock_arith.h).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
if_present=0
stock=0
while [ $# -gt 0 ]; do
  case "$1" in
    --if-present) if_present=1; shift ;;
    --stock) stock=1; shift ;;
    *) break ;;
  esac
done
ref="${1:-${RILS_ROLS_REFERENCE:-/root/reference}}"
src="$ref/rils_rols_cpp"
if [ ! -f "$src/rils_rols_cpp.cpp" ]; then
  if [ "$if_present" = 1 ]; then echo "no reference checkout at $ref: reference harness not built"; exit 0; fi
  echo "reference sources not found under $src" >&2; exit 3
fi
mkdir -p "$here/_ref"
pyinc="$(python3 -c 'import pybind11,sysconfig;print("-I"+pybind11.get_include()+" -I"+sysconfig.get_paths()["include"])')"
# -ffp-contract=off: no implicit FMA contraction (the explicit fma() calls of the
# fixed-order sums stay), so x86 and Arm builds round alike.
out="$here/_ref/librr_ref.so"
[ "$stock" = 1 ] && out="$here/_ref/librr_ref_stock.so"
# up to date: newer than every source it is made from
fresh=1
for f in "$src/rils_rols_cpp.cpp" "$src/node.cpp" "$src/node.h" "$here/ref_harness.cpp" "$here/colpiv_qr.h" \
         "$here/eigen_shim/"* "$here/../rils-rols_gb300/csrc/common/rr_math.h" \
         "$here/../rils-rols_gb300/csrc/common/rr_sum.h" "$0"; do
  [ "$out" -nt "$f" ] || fresh=0
done
if [ "$fresh" = 1 ]; then echo "up to date: $out"; exit 0; fi
if [ "$stock" = 1 ]; then
  g++ -std=c++17 -march=native -O3 -fPIC -shared -w \
      -include "$here/eigen_shim/stock_arith.h" -include "$here/eigen_shim/rr_module_guards.h" \
      -I "$here/eigen_shim" -I "$src" $pyinc \
      "$here/ref_harness.cpp" "$src/node.cpp" -o "$here/_ref/librr_ref_stock.so"
  echo "built $here/_ref/librr_ref_stock.so"
  exit 0
fi
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w \
    -include "$here/eigen_shim/rr_module_guards.h" -I "$here/eigen_shim" -I "$src" $pyinc \
    "$here/ref_harness.cpp" "$src/node.cpp" -o "$here/_ref/librr_ref.so"
echo "built $here/_ref/librr_ref.so"
