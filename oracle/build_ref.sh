#!/bin/sh
# Builds the reference library's own headers (header-only C++) through
# ref_driver.cpp into oracle/_ref/. TEST INFRASTRUCTURE AND CPU BASELINE
# ONLY: the tests pin the C restatement (intp_oracle.c) against it, the
# golden-fixture script records its outputs, and the benchmark's reference
# arm times it on the host cores. Nothing in the product loads it.
#
# Headers: $INTP_REFERENCE_INCLUDE, else $INTP_REFERENCE_ROOT/src/include,
# else the staged install baseline/_ref/include (oracle/stage_ref.sh). Skips
# quietly when none exists.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REPO=$(dirname "$HERE")
INC=${INTP_REFERENCE_INCLUDE:-}
if [ -z "$INC" ] && [ -n "$INTP_REFERENCE_ROOT" ]; then INC="$INTP_REFERENCE_ROOT/src/include"; fi
if [ -z "$INC" ]; then INC="$REPO/baseline/_ref/include"; fi
if [ ! -f "$INC/Interpolation.hpp" ]; then
    echo "reference headers not found ($INC); oracle/_ref not built"
    exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXX=${CXX:-g++}
# the reference's own flags for its multithreaded build: the 8-thread pool of
# the solve (INTP_MULTITHREAD), periodic axes without the dummy point
FLAGS="-std=c++17 -O3 -fPIC -shared -ffp-contract=off -DINTP_MULTITHREAD -DINTP_PERIODIC_NO_DUMMY_POINT -I$INC"
# plain control-point layout (control points readable in row-major order)
$CXX $FLAGS "$HERE/ref_driver.cpp" -o "$OUT/libintp_ref_plain.so.tmp" -lpthread &
# the reference test build's layout (test/CMakeLists.txt:46-47)
$CXX $FLAGS -DINTP_CELL_LAYOUT "$HERE/ref_driver.cpp" -o "$OUT/libintp_ref_cell.so.tmp" -lpthread &
wait
mv "$OUT/libintp_ref_plain.so.tmp" "$OUT/libintp_ref_plain.so"
mv "$OUT/libintp_ref_cell.so.tmp" "$OUT/libintp_ref_cell.so"
echo "built $OUT from $INC"
