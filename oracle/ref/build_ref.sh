#!/usr/bin/env bash
# Test infrastructure: compiles the reference's own path-tracer sources (read in place from
# the reference checkout, never copied) into the host program oracle/_ref/lts_ref.
#   g++ -E (shim force-included)  |  instrument.pl (launch rewrite + recording hooks)  |  g++
# Needs only g++ with OpenMP.  Usage: oracle/ref/build_ref.sh [REFERENCE_ROOT]
set -euo pipefail
REF="${1:-${LTS_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/../_ref"
if [ ! -f "$REF/src/acceleration/BVH.cuh" ]; then
    echo "build_ref.sh: reference sources not found under $REF" >&2
    exit 4
fi
mkdir -p "$OUT"
g++ -E -std=c++17 -DNDEBUG -fopenmp -I"$HERE/shim/include" -include "$HERE/shim/lts_ref_shim.h" \
    -I"$REF/src" "$HERE/ref_unity.cpp" \
  | perl "$HERE/instrument.pl" \
  | g++ -x c++ -std=c++17 -O2 -fopenmp -ffp-contract=off -fpermissive -w -o "$OUT/lts_ref.tmp" -
mv "$OUT/lts_ref.tmp" "$OUT/lts_ref"
echo "built $OUT/lts_ref"
