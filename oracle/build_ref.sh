#!/usr/bin/env bash
# Compile the reference's own soup fast-winding-number code (header-only,
# Eigen-free: FastWindingNumberForSoups.h + parallel_for.h +
# default_num_threads) straight from the reference tree into oracle/_ref/.
# Runs only where the reference tree exists; outputs never enter git history.
# Test infrastructure only (pinning + golden-fixture generation).
set -euo pipefail
# The libigl source tree is named by GWN_REFERENCE_ROOT (no default).
REF="${GWN_REFERENCE_ROOT:-}"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ -z "$REF" ] || [ ! -f "$REF/include/igl/FastWindingNumberForSoups.h" ]; then
  echo "reference tree not present at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
ARCHFLAGS=""
case "$(uname -m)" in x86_64) ARCHFLAGS="-msse4.1" ;; esac
g++ -O3 -std=c++17 $ARCHFLAGS -w -fPIC -shared -I"$REF/include" \
  "$HERE/ref_soup_wrap.cpp" -o "$HERE/_ref/libref_soup.so" -lpthread
echo "built $HERE/_ref/libref_soup.so"
