#!/bin/sh
# Compile the reference project's own CPU code (its complex128 oracle, plan
# builder, Pauli helpers and circuit generators) straight from its sources,
# plus ref_shim.cpp, into oracle/_ref/libqref.so. Test infrastructure only.
#
#   QMETAL_REFERENCE_SRC=/path/to/reference sh oracle/build_ref.sh
#   sh oracle/build_ref.sh --where   # print the source tree it would use
#
# The reference tree is QMETAL_REFERENCE_SRC (REF is accepted too), else the
# location this build environment mounts it at. Exit status 3 when there is
# no tree there. Reads the sources where they lie; writes only under
# oracle/_ref/.
set -e
REF="${QMETAL_REFERENCE_SRC:-${REF:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/reference.cpp" ]; then
  echo "build_ref: reference sources not found at $REF" >&2
  exit 3
fi
if [ "$1" = "--where" ]; then
  echo "$REF"
  exit 0
fi
mkdir -p "$OUT"
g++ -std=c++17 -O2 -fPIC -shared -I"$REF/include" \
    "$REF/src/reference.cpp" "$REF/src/plan.cpp" "$REF/src/pauli.cpp" \
    "$REF/src/circuits.cpp" "$HERE/ref_shim.cpp" -o "$OUT/libqref.so.tmp"
mv "$OUT/libqref.so.tmp" "$OUT/libqref.so"
echo "build_ref: wrote $OUT/libqref.so"
