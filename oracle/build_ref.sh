#!/usr/bin/env bash
# ORACLE build recipe (test infrastructure only).
# Compiles the reference's own sources, unmodified and where they lie, into
# oracle/_ref/librr_ref.so, against the self-written Eigen subset in
# oracle/eigen_shim/ (the vendored Eigen lacks Eigen/Core).  Runs only where
# the reference checkout exists; the GPU host never builds or loads this.
#   usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-/root/reference}"
src="$ref/rils_rols_cpp"
[ -f "$src/rils_rols_cpp.cpp" ] || { echo "reference sources not found under $src" >&2; exit 3; }
mkdir -p "$here/_ref"
pyinc="$(python3 -c 'import pybind11,sysconfig;print("-I"+pybind11.get_include()+" -I"+sysconfig.get_paths()["include"])')"
# -ffp-contract=off: no implicit FMA contraction (the explicit fma() calls of the
# fixed-order sums stay), so x86 and Arm builds round alike.
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w \
    -include "$here/eigen_shim/rr_module_guards.h" -I "$here/eigen_shim" -I "$src" $pyinc \
    "$here/ref_harness.cpp" "$src/node.cpp" -o "$here/_ref/librr_ref.so"
echo "built $here/_ref/librr_ref.so"
