#!/usr/bin/env bash
# Build recipe for oracle/_ref: compiles glsCV's own CPU Stockham source
# (UnitTest_glsCV/fft_stockhum.cpp) from the read-only reference checkout into
# oracle/_ref/libref_stockham.so, for validating the C restatement in
# oracle/stockham.c.  Test infrastructure only.
#
# Two build-time adjustments, applied to a temporary copy (the patched source
# is never written into this repository):
#   1. `#include "stdafx.h"` resolves to oracle/ref_shim/stdafx.h (a tiny
#      cv::Mat stand-in; OpenCV is not available here).
#   2. `n = n++` -> `n++` in the butterfly loops: under g++ that statement
#      leaves n unchanged, so those loops would never end.
#
# Usage: oracle/build_ref.sh REFERENCE_ROOT   (or GLS_REFERENCE_ROOT set)
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-${GLS_REFERENCE_ROOT:-}}"
if [ -z "$ref" ]; then
    echo "build_ref: pass the glsCV checkout or set GLS_REFERENCE_ROOT" >&2
    exit 2
fi
src="$ref/UnitTest_glsCV/fft_stockhum.cpp"
out="$here/_ref"
if [ ! -f "$src" ]; then
    echo "build_ref: $src not found; oracle/_ref not built" >&2
    exit 2
fi
mkdir -p "$out"
tmp="$(mktemp -d)"
trap 'rm -rf "$tmp"' EXIT
sed -e 's/n = n++/n++/g' "$src" > "$tmp/fft_stockhum_ref.cpp"
# same flags as oracle/stockham.c: no FMA contraction, so the restatement and
# the reference round identically
flags="-std=c++14 -O2 -fPIC -fopenmp -ffp-contract=off -w"
g++ $flags -I"$here/ref_shim" -c "$tmp/fft_stockhum_ref.cpp" -o "$tmp/fft_stockhum_ref.o"
g++ $flags -I"$here/ref_shim" -c "$here/ref_shim/ref_wrap.cpp" -o "$tmp/ref_wrap.o"
g++ -shared -fopenmp -o "$out/libref_stockham.so" "$tmp/fft_stockhum_ref.o" "$tmp/ref_wrap.o"
echo "build_ref: built $out/libref_stockham.so"
