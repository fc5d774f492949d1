#!/bin/sh
# Stages the reference library's headers (12ff54e/BSplineInterpolation,
# src/include, header-only C++) into baseline/_ref/include: the reference
# install that the benchmark's reference arm and oracle/build_ref.sh compile
# against. baseline/_ref is git-ignored (never committed); it travels with
# the working tree to the GPU host, which has no reference tree of its own.
# The reference is a CMake INTERFACE library with no Python packaging, so a
# copy of its include directory is its whole install.
#
#   sh oracle/stage_ref.sh <reference root>     (or INTP_REFERENCE_ROOT=<root>)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REPO=$(dirname "$HERE")
REF=${1:-$INTP_REFERENCE_ROOT}
if [ -z "$REF" ] || [ ! -f "$REF/src/include/Interpolation.hpp" ]; then
    echo "usage: sh oracle/stage_ref.sh <reference root> (src/include/Interpolation.hpp not found)" >&2
    exit 2
fi
DEST="$REPO/baseline/_ref/include"
mkdir -p "$DEST"
cp "$REF"/src/include/*.hpp "$DEST/"
echo "staged $(ls "$DEST" | wc -l) headers into $DEST"
