#!/usr/bin/env bash
# Builds the reference WeldFormFEM CPU path, read in place from the reference
# checkout, into oracle/_ref/libwfref.so together with oracle/ref_harness.cpp.
# TEST INFRASTRUCTURE ONLY: the result is the oracle the restated C oracle and
# the golden fixtures are checked against; the product never links it.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default: $WF_REFERENCE_ROOT)
# Outputs go only to oracle/_ref/ (git-ignored). The reference's own CMake is
# not used: it requires SCOTCH and the empty git submodules. Two stub headers
# (oracle/ref_stubs/) stand in for the missing LS-DYNA reader submodule and the
# CMake-generated git_commit.h.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${WF_REFERENCE_ROOT:-}}"
if [ -z "$REF" ] || [ ! -f "$REF/src/common/Domain_d.C" ]; then
  echo "build_ref.sh: reference checkout not found (pass its root as \$1)" >&2
  exit 2
fi
OUT="$HERE/_ref"
mkdir -p "$OUT/obj"
CXX="${CXX:-g++}"
# -ffp-contract=off keeps the reference's intent of no FMA contraction
# (src/common/CMakeLists.txt:16 passes --fmad=false to nvcc).
FLAGS="-x c++ -std=c++17 -O2 -fopenmp -ffp-contract=off -fPIC -w"
INC="-I$REF/include/common -I$REF/include -I$REF/src/common -I$HERE/ref_stubs/include -I$HERE/ref_stubs/lib/LSDynaReader/src"
SRCS="src/common/Domain_d.C src/common/Mechanical.C src/common/Matrices.C src/common/Contact.C src/common/Mesh.C src/common/VTKWriter.C src/common/Thermal.C src/explicit/Solver_explicit.C"
pids=()
for f in $SRCS; do
  b=$(basename "$f" .C)
  $CXX $FLAGS $INC -c "$REF/$f" -o "$OUT/obj/$b.o" &
  pids+=($!)
done
$CXX $FLAGS $INC -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
$CXX -shared -fopenmp -o "$OUT/libwfref.so" "$OUT"/obj/*.o
echo "built $OUT/libwfref.so"
