#!/bin/sh
# Builds the reference's own C++/OpenMP MEX kernels (from the read-only
# SGLDBench checkout, unmodified) against the oracle's MEX shim, into
# oracle/_ref/libref_mex.so.  Each file's mexFunction is renamed to
# ref_<file stem> so that the kernels can live in one library.
# Test infrastructure only: the product never links or loads this library.
set -e
REF=${SGLD_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SRC="$REF/src/MEXfuncs"
[ -d "$SRC" ] || { echo "reference sources not found at $SRC (set SGLD_REFERENCE)" >&2; exit 2; }
mkdir -p "$OUT/obj"
CXX=${CXX:-g++}
FLAGS="-O3 -fopenmp -fPIC -std=c++17 -w -I$HERE/mexshim"
OBJS=""
for f in Solving_KbyU_MatrixFree_mex Solving_Restriction_MatrixFree_mex \
         Solving_Interpolation_MatrixFree_mex Solving_AssembleCmptStencilFromFinestLevel \
         Solving_AssembleCmptStencilFromNonFinestLevel TopOpti_CmptUnitCompliance_mex \
         TopOpti_SetupDensityFilter_mex TopOpti_PerformDensityFiltering_mex \
         Solving_KbyU_MatrixFree8x8_mex; do
  $CXX $FLAGS -DmexFunction=ref_$f -c "$SRC/$f.cpp" -o "$OUT/obj/$f.o" &
  OBJS="$OBJS $OUT/obj/$f.o"
done
# MMA: the gateway and the solver class it instantiates
$CXX $FLAGS -I"$SRC" -DmexFunction=ref_MMA_mex -c "$SRC/MMA_mex.cpp" -o "$OUT/obj/MMA_mex.o" &
$CXX $FLAGS -I"$SRC" -c "$SRC/MMAseq.cpp" -o "$OUT/obj/MMAseq.o" &
OBJS="$OBJS $OUT/obj/MMA_mex.o $OUT/obj/MMAseq.o"
$CXX $FLAGS -c "$HERE/mexshim/mexshim.cpp" -o "$OUT/obj/mexshim.o" &
wait
$CXX -shared -fopenmp -o "$OUT/libref_mex.so" $OBJS "$OUT/obj/mexshim.o"
# record where the checkout is, for the tests that read its data files
(cd "$REF" && pwd) > "$OUT/REFERENCE_ROOT"
echo "built $OUT/libref_mex.so"
