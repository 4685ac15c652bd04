#!/usr/bin/env bash
# Builds oracle/_ref/ref_harness from the reference's own headers where they
# lie (read-only source tree, nothing copied), against oracle/eigen_subset.
# Test infrastructure only; the output directory is git-ignored.
# usage: oracle/build_ref.sh REFERENCE_ROOT   (or METADA_REFERENCE set)
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ref="${1:-${METADA_REFERENCE:-}}"
if [ -z "$ref" ]; then
  echo "usage: $0 REFERENCE_ROOT (or set METADA_REFERENCE); ref_harness not built" >&2
  exit 2
fi
if [ ! -d "$ref/src" ]; then
  echo "reference tree not found at $ref; ref_harness not built" >&2
  exit 3
fi
mkdir -p "$here/_ref"
incs=(-I "$here/eigen_subset")
# Only the directories on the analysis path: other backends (Lorenz-63, WRF,
# Lite, gmock) define headers with the same names.
for d in traits framework/base framework/algorithms framework/adapters \
         framework/adapters/common/utils/config framework/adapters/common/utils/logger \
         backends/simple backends/common/observation backends/common/obsoperator \
         backends/common/utils/logger/console; do
  incs+=(-I "$ref/src/$d")
done
# SimpleState.hpp calls std::min_element without including <algorithm>.
g++ -std=c++20 -O2 -ffp-contract=off -include algorithm -include numeric -w \
  -I "$here" "${incs[@]}" "$here/ref_harness.cpp" -o "$here/_ref/ref_harness"
echo "built $here/_ref/ref_harness"
