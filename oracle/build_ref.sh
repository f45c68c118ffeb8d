#!/bin/sh
# Compile the reference's serial and OpenMP pricing sources, where they lie,
# into oracle/_ref/ref_<name>.so (one shared object per source file, because
# the reference's include/common.h defines non-inline functions).
#
# TEST INFRASTRUCTURE ONLY. The objects are the checker's pin: the golden
# fixtures in tests/golden/ref_outputs.json are their outputs. Reference
# sources are read in place and never copied. mc_eur_multi* needs Eigen and
# Boost, which this image does not have, so it is not built.
#
# Usage: sh oracle/build_ref.sh REFERENCE_ROOT
#        (or PCF_REFERENCE_ROOT=... sh oracle/build_ref.sh)
set -e
REF=${1:-$PCF_REFERENCE_ROOT}
[ -n "$REF" ] || { echo "usage: $0 REFERENCE_ROOT"; exit 2; }
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -d "$REF/src" ] || { echo "reference not found at $REF; skipping"; exit 0; }
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-O2 -std=c++17 -fopenmp -fPIC -ffp-contract=off -w -I$HERE/ref_stub -I$REF/include"
build() { # name fn kind
  $CXX $FLAGS -Dmain=ref_unused_main_$1 -c "$REF/src/$1.cpp" -o "$OUT/$1.o"
  $CXX $FLAGS -DREF_FN=$2 -DREF_KIND=$3 -c "$HERE/ref_stub/ref_shim.cpp" -o "$OUT/$1_shim.o"
  $CXX -shared -fopenmp -Wl,-Bsymbolic -o "$OUT/ref_$1.so" "$OUT/$1.o" "$OUT/$1_shim.o"
  rm -f "$OUT/$1.o" "$OUT/$1_shim.o"
}
build mc_eur mc_eur 1 &
build mc_eur_omp mc_eur 1 &
build mc_asia mc_asia 2 &
build mc_asia_omp mc_asia 2 &
build mc_amer mc_amer 2 &
build mc_amer_omp mc_amer 3 &
build binom_embar binom 1 &
build binom_embar_omp binom 1 &
build binom_vanilla_eur binom 1 &
build binom_vanilla_amer binom 1 &
wait
ls "$OUT"
