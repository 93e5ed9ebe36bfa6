#!/usr/bin/env bash
# Compiles the lbmminiapp reference's serial CPU sources, unmodified and where
# they lie, together with oracle/ref_harness.cpp and the single-rank MPI stub,
# into oracle/_ref/libref_q19.so and oracle/_ref/libref_q27.so.
#
# Test infrastructure only (the oracle): the outputs are git-ignored and are
# used by tests/ to pin oracle/lbm_oracle.c and the golden fixtures against
# the reference itself.  Needs the reference sources; exits 0 without building
# when they are absent.  The sources are looked up in $LBM_REFERENCE_DIR, else in
# a checkout named "reference" beside this repository.
#
#   -DSOA                 : the population layout the hot path uses
#   -D_LATTICESIZE_=19|27 : one library per lattice (src/Parameters.hh:6-8)
#   -ffp-contract=off     : IEEE double arithmetic without FMA contraction, so
#                           x86-64 and aarch64 builds give the same bits
#   -include ref_overrides.h : run-time _OMEGA_ / _GRAVITY_ (see that header)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${LBM_REFERENCE_DIR:-$(cd "$HERE/../.." && pwd)/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF/src/kernels" ]; then
  echo "build_ref: reference sources not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
SRC="$REF/src"
INC="-I$HERE/mpi_stub -I$SRC -I$SRC/geometries -I$SRC/kernels -I$SRC/lattices -I$SRC/propagation"
FILES="$SRC/Parameters.cpp $SRC/Communication.cpp
  $SRC/geometries/Geometry.cpp $SRC/geometries/GeometryAAAB.cpp
  $SRC/lattices/LatticeD3Q19.cpp $SRC/lattices/LatticeD3Q27.cpp
  $SRC/propagation/Propagation.cpp $SRC/propagation/PropagationAA.cpp $SRC/propagation/PropagationAB.cpp
  $SRC/kernels/KernelAA_SOA_Base.cpp $SRC/kernels/KernelAA_SOA_Unroll.cpp $SRC/kernels/KernelAA_AOS_Base.cpp
  $SRC/kernels/KernelAB_SOA_Base.cpp $SRC/kernels/KernelAB_SOA_Unroll.cpp
  $SRC/kernels/KernelAB_SOA_Pull.cpp $SRC/kernels/KernelAB_SOA_Unroll_Pull.cpp $SRC/kernels/KernelAB_AOS_Base.cpp
  $HERE/ref_harness.cpp"
CXX="${CXX:-g++}"
for Q in 19 27; do
  "$CXX" -O2 -std=c++17 -fPIC -shared -ffp-contract=off -w -DSOA -D_LATTICESIZE_=$Q \
    -include "$HERE/ref_overrides.h" $INC $FILES -o "$OUT/libref_q$Q.so.tmp" &
done
wait
for Q in 19 27; do mv "$OUT/libref_q$Q.so.tmp" "$OUT/libref_q$Q.so"; done
echo "build_ref: built $OUT/libref_q19.so $OUT/libref_q27.so"
