#!/bin/sh
# Builds the reference library's own headers (header-only C++, read in place,
# never copied) through ref_driver.cpp into oracle/_ref/. Test infrastructure:
# used to pin the C oracle and to record golden fixtures. Skips quietly when
# the reference tree is absent (it is not present on GPU hosts).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${INTP_REFERENCE_ROOT:-/root/reference}
if [ ! -f "$REF/src/include/Interpolation.hpp" ]; then
    echo "reference headers not found at $REF; oracle/_ref not built"
    exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-std=c++17 -O3 -fPIC -shared -ffp-contract=off -DINTP_MULTITHREAD -DINTP_PERIODIC_NO_DUMMY_POINT -I$REF/src/include"
# plain control-point layout (control points readable in row-major order)
$CXX $FLAGS "$HERE/ref_driver.cpp" -o "$OUT/libintp_ref_plain.so" -lpthread &
# the reference test build's layout (test/CMakeLists.txt:46-47)
$CXX $FLAGS -DINTP_CELL_LAYOUT "$HERE/ref_driver.cpp" -o "$OUT/libintp_ref_cell.so" -lpthread &
wait
echo "built $OUT"
