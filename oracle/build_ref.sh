#!/usr/bin/env bash
# Build the reference's own permanent calculators (compiled from their sources
# where they lie in the reference tree; nothing is copied) together with the
# TBB stand-in in oracle/tbbshim and the C entry points in oracle/ref_capi.cpp.
# Output: oracle/_ref/libpqbref.so.  Oracle-only; runs where the reference tree
# is present (the development container), never in the product build.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${PQB_REFERENCE_ROOT:-/root/reference}/piquassoboost"
if [ ! -d "$REF/sampling/source" ]; then
  echo "reference tree not found at $REF; skipping oracle/_ref" >&2
  exit 3
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
C="$REF/common/source"
S="$REF/sampling/source"
SRCS=(
  "$C/matrix.cpp" "$C/matrix32.cpp" "$C/PicState.cpp" "$C/common_functionalities.cpp"
  "$C/n_aryGrayCodeCounter.cpp" "$C/PicTypes.cpp"
  "$S/BBFGPermanentCalculator.cpp" "$S/BBFGPermanentCalculatorRepeated.cpp"
  "$S/GlynnPermanentCalculators_implementation.cpp" "$S/GlynnPermanentCalculatorSimple.cpp"
  "$S/CChinHuhPermanentCalculator.cpp" "$S/BatchedPermanentCalculator.cpp"
  "$REF/sampling/simulation_strategies/source/samplingHelperFunctions.cpp"
  "$REF/sampling/simulation_strategies/source/CGeneralizedCliffordsBSimulationStrategy.cpp"
  "$REF/sampling/simulation_strategies/source/CGeneralizedCliffordsBUniformLossesSimulationStrategy.cpp"
  "$HERE/ref_capi.cpp"
)
OBJS=()
pids=()
for s in "${SRCS[@]}"; do
  o="$OUT/$(basename "${s%.cpp}").o"
  OBJS+=("$o")
  g++ -std=c++17 -O3 -fPIC -DBLAS=3 -w -I "$HERE/tbbshim" -I "$C" -I "$S" \
      -I "$REF/sampling/simulation_strategies/source" -c "$s" -o "$o" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libpqbref.so" "${OBJS[@]}" -lpthread
rm -f "${OBJS[@]}"
echo "built $OUT/libpqbref.so"
