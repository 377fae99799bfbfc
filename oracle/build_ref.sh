#!/bin/sh
# Compile the reference project's own CPU code (its complex128 oracle, plan
# builder, Pauli helpers and circuit generators) straight from its sources,
# plus ref_shim.cpp, into oracle/_ref/libqref.so. Test infrastructure only.
#
#   REF=/path/to/reference sh oracle/build_ref.sh
#
# Reads the sources where they lie; writes only under oracle/_ref/.
set -e
REF="${REF:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/reference.cpp" ]; then
  echo "build_ref: reference sources not found at $REF" >&2
  exit 1
fi
mkdir -p "$OUT"
g++ -std=c++17 -O2 -fPIC -shared -I"$REF/include" \
    "$REF/src/reference.cpp" "$REF/src/plan.cpp" "$REF/src/pauli.cpp" \
    "$REF/src/circuits.cpp" "$HERE/ref_shim.cpp" -o "$OUT/libqref.so.tmp"
mv "$OUT/libqref.so.tmp" "$OUT/libqref.so"
echo "build_ref: wrote $OUT/libqref.so"
