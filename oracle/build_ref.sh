#!/usr/bin/env bash
# Compile the reference's own hot-path sources, unmodified and where they lie, against the
# one-rank shims in oracle/ref_shim, into oracle/_ref/libref_nvar{5,7,9,11,15}.so, and its IMEX
# program's chemistry-hydrodynamics glue into oracle/_ref/libref_glue.so.
#
# TEST INFRASTRUCTURE ONLY: the result checks the oracle restatement (oracle/oracle.c) and
# generates tests/golden/*.npz.  It needs the reference tree, so it runs only where that tree
# exists; usage:  oracle/build_ref.sh [REFERENCE_ROOT]
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-${GBMV_REFERENCE_ROOT:-/root/reference}}"
src="$ref/src"
if [ ! -f "$src/utilities.cpp" ]; then
  echo "build_ref.sh: reference sources not found under $ref" >&2
  exit 2
fi
out="$here/_ref"
mkdir -p "$out"
shim="$here/ref_shim"
CXX="${CXX:-g++}"
CC="${CC:-gcc}"
# -ffp-contract=off: no FMA contraction, so the reference's arithmetic is evaluated as written.
flags="-O2 -fPIC -ffp-contract=off -DRAJA_SERIAL -DUSEHDF5 -w"
$CC -O2 -fPIC -ffp-contract=off -c "$shim/shim_impl.c" -o "$out/shim_impl.o"
pids=()
for nv in 5 7 9 11 15; do
  (
    $CXX -std=c++14 $flags -DNVAR=$nv -I"$shim" -I"$src" -shared -o "$out/libref_nvar$nv.so" \
      "$here/ref_driver.cpp" "$src/utilities.cpp" "$src/raja_primordial_network.cpp" \
      "$out/shim_impl.o"
  ) &
  pids+=($!)
done
# the chemistry-hydrodynamics glue of the IMEX program (fexpl, PostprocessStep) with the static
# problem's Dengo-scaling routines, NVAR 15 (oracle/ref_glue.cpp includes the program's file)
(
  $CC -O2 -fPIC -ffp-contract=off -I"$shim" -c "$shim/shim_glue.c" -o "$out/shim_glue.o"
  $CXX -std=c++14 $flags -DNVAR=15 -I"$shim" -I"$src" -shared -o "$out/libref_glue.so" \
    "$here/ref_glue.cpp" "$src/primordial_static.cpp" "$src/utilities.cpp" \
    "$src/raja_primordial_network.cpp" "$out/shim_impl.o" "$out/shim_glue.o"
) &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
echo "built: $(ls "$out"/*.so | tr '\n' ' ')"
