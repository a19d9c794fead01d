#!/bin/sh
# Builds oracle/_ref/libbirp_ref.so from the UNMODIFIED reference sources
# where they lie (src/Camera.cpp, DataCube.cpp, Cmem.cpp, Helper.cpp), plus
# the no-op EleFits headers in oracle/ref_shim and the C wrappers
# oracle/ref_capi.cpp and oracle/helper_shim.cpp. Test infrastructure only (pins the oracle and makes the
# golden fixtures).
#
# Usage: build_ref.sh <reference project directory>   (or BIRP_REFERENCE_DIR=<dir>)
# Without a directory that holds the reference sources it builds nothing and
# exits 0, so a machine without the reference tree skips it.
set -e
REF=${1:-$BIRP_REFERENCE_DIR}
if [ -z "$REF" ]; then
  echo "no reference directory given (argument or BIRP_REFERENCE_DIR); skipping oracle/_ref" >&2
  exit 0
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/src/Camera.cpp" ]; then
  echo "reference sources not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
# Same optimisation level as the reference's own Release build (-O3, C++23);
# no -march, so no FMA contraction on x86-64.
g++ -O3 -std=c++23 -fPIC -shared -w \
  -I"$HERE/ref_shim" -I"$REF/include" \
  "$REF/src/Camera.cpp" "$REF/src/DataCube.cpp" "$REF/src/Cmem.cpp" "$REF/src/Helper.cpp" \
  "$HERE/ref_capi.cpp" "$HERE/helper_shim.cpp" -o "$OUT/libbirp_ref.so"
echo "built $OUT/libbirp_ref.so"
