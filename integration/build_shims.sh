#!/usr/bin/env bash
# Compiles the reference-side shims (integration/*.hh, driven by
# integration/shim_check.cpp) against the UNMODIFIED lbmminiapp headers and
# sources, where they lie, and links them to lbmminiapp_gb300/liblbm_gb300.so:
# oracle/_ref/libgb300_shims_q19.so and libgb300_shims_q27.so (git-ignored).
# This is the build a maintainer's Makefile would do after adding the shims to
# the reference (-DSOA, one library per _LATTICESIZE_, the single-rank MPI stub
# of oracle/mpi_stub in place of an MPI installation).  Needs the reference
# sources ($LBM_REFERENCE_DIR, else a checkout named "reference" beside this
# repository) and the built library; exits 0 without building when the sources
# are absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ROOT="$(cd "$HERE/.." && pwd)"
REF="${LBM_REFERENCE_DIR:-$(cd "$ROOT/.." && pwd)/reference}"
OUT="$ROOT/oracle/_ref"
LIBDIR="$ROOT/lbmminiapp_gb300"
if [ ! -d "$REF/src/kernels" ]; then
  echo "build_shims: reference sources not found at $REF; skipping" >&2
  exit 0
fi
[ -f "$LIBDIR/liblbm_gb300.so" ] || { echo "build_shims: build lbmminiapp_gb300/liblbm_gb300.so first" >&2; exit 1; }
mkdir -p "$OUT"
SRC="$REF/src"
INC="-I$ROOT/include -I$HERE -I$ROOT/oracle/mpi_stub -I$SRC -I$SRC/geometries -I$SRC/kernels -I$SRC/lattices -I$SRC/propagation"
FILES="$SRC/Parameters.cpp $SRC/Communication.cpp
  $SRC/geometries/Geometry.cpp $SRC/geometries/GeometryAAAB.cpp
  $SRC/lattices/LatticeD3Q19.cpp $SRC/lattices/LatticeD3Q27.cpp
  $SRC/propagation/Propagation.cpp
  $HERE/shim_check.cpp"
CXX="${CXX:-g++}"
pids=()
for Q in 19 27; do
  "$CXX" -O2 -std=c++17 -fPIC -shared -Wall -Wno-unused-variable -Wno-sign-compare -Wno-unused-but-set-variable \
    -DSOA -D_LATTICESIZE_=$Q $INC $FILES -L"$LIBDIR" -llbm_gb300 -Wl,-rpath,"$LIBDIR" \
    -o "$OUT/libgb300_shims_q$Q.so.tmp" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
for Q in 19 27; do mv "$OUT/libgb300_shims_q$Q.so.tmp" "$OUT/libgb300_shims_q$Q.so"; done
echo "build_shims: built $OUT/libgb300_shims_q19.so $OUT/libgb300_shims_q27.so"
