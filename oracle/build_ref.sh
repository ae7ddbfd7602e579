#!/usr/bin/env bash
# Builds the reference solver's CPU code, unmodified, from its own sources, plus the dump
# harness (oracle/ref_harness.cpp) into oracle/_ref/ref_harness. Test infrastructure only.
#
# Flags: FP64 build (-DSINGLE: the reference's REAL is double only when SINGLE is defined),
# no FP contraction so results do not depend on FMA formation, BL_Model.cpp without OpenMP
# (GCC rejects its firstprivate loop variables). source/TimeStep.cpp is UTF-16 and is
# converted into the output directory before compiling. Runs with NT=1 only.
#
#   oracle/build_ref.sh [REF_ROOT]
#
# REF_ROOT is the reference checkout (the argument, else the REF_ROOT environment variable, else a
# directory named "reference" beside this repository). FP32=1 builds the reference's default FP32
# build (REAL = float) into oracle/_ref32 instead.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${REF_ROOT:-$HERE/../../reference}}"
OUT="$HERE/_ref"
PREC="-DSINGLE"
if [ "${FP32:-0}" = "1" ]; then
  OUT="$HERE/_ref32"
  PREC=""
fi
if [ ! -d "$REF/source" ]; then
  echo "reference sources not found at $REF (the oracle/_ref build only runs where they exist)" >&2
  exit 3
fi
mkdir -p "$OUT/obj"
iconv -f UTF-16 -t UTF-8 "$REF/source/TimeStep.cpp" > "$OUT/TimeStep_utf8.cpp"
CXX="${CXX:-g++}"
FLAGS="-std=c++17 -O2 -fpermissive -w $PREC -D_finite=finite -D_isnan=isnan -ffp-contract=off -I$REF/include"
pids=()
for src in "$REF"/source/*.cpp "$OUT/TimeStep_utf8.cpp"; do
  base="$(basename "$src" .cpp)"
  case "$base" in
    Structured_FV3D|TimeStep) continue ;;   # driver main replaced by the harness; UTF-16 original
  esac
  omp="-fopenmp"
  [ "$base" = "BL_Model" ] && omp=""
  $CXX $FLAGS $omp -c "$src" -o "$OUT/obj/$base.o" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
$CXX $FLAGS -Dprivate=public -fopenmp -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o"
$CXX -fopenmp "$OUT"/obj/*.o -o "$OUT/ref_harness"
echo "built $OUT/ref_harness"
