#!/usr/bin/env bash
# Builds oracle/_ref/librace_ref.so: the RACE reference library compiled in
# place from its own sources (the SOURCES list of the reference's
# CMakeLists.txt:23-42) plus oracle/ref_capi.cpp, with the shims in
# oracle/shim standing in for the un-vendored GAP headers, hwloc and the
# CMake-generated config.h. Nothing is copied out of the reference tree.
# Flags: -O3 without -Ofast and with -ffp-contract=off, so the reference's
# double arithmetic in the load balancer is plain IEEE.
# The reference uses x86 intrinsics (_mm_pause) in its executor, so this
# build is x86-only; it is test infrastructure for generating golden data.
set -euo pipefail
REF="${RACE_REFERENCE_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
mkdir -p "$OUT/obj"
[ -d "$REF/src" ] || { echo "reference sources not found at $REF" >&2; exit 2; }
SRCS="graph traverse levelData lb error zone_tree level_recursion interface functionManager machine pin level_pool dummy signal sell_c_sigmize matrixPower matrixPowerRecursive"
CXXFLAGS="-O3 -fopenmp -std=c++17 -fPIC -ffp-contract=off -w -I$HERE/shim -I$REF/include -D'kmp_set_warnings_off()=((void)0)'"
pids=()
for s in $SRCS; do
  eval g++ $CXXFLAGS -c "$REF/src/$s.cpp" -o "$OUT/obj/$s.o" &
  pids+=($!)
done
eval g++ $CXXFLAGS -c "$HERE/ref_capi.cpp" -o "$OUT/obj/ref_capi.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -fopenmp -o "$OUT/librace_ref.so" "$OUT"/obj/*.o
echo "built $OUT/librace_ref.so"
