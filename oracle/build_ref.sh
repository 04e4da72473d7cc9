#!/usr/bin/env bash
# Builds the reference AnsatzEvolve library (real and complex variants) straight from
# its own sources, plus the pinning driver oracle/ref_driver.cpp, into oracle/_ref/.
# Test infrastructure only: oracle/_ref/ validates the C restatement in
# oracle/oracle.c and produces the golden fixtures under tests/golden/.
# The reference's CMake project needs gfortran, so the translation units are
# compiled directly.  Needs the reference checkout: AE_REFERENCE, else a `reference`
# directory beside this repository.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${AE_REFERENCE:-$HERE/../../reference}/src
OUT=$HERE/_ref
[ -d "$REF" ] || { echo "reference sources not found at $REF" >&2; exit 2; }
mkdir -p "$OUT/obj_real" "$OUT/obj_cplx"
SRCS="AnsatzManager AnsatzSynthInterface TUPSLoadingUtils ansatz benchmark csvwriter diis
      fusedevolve hamiltonianmatrix linalg logger operatorpool sparsematrix threadpool tupsquantities"
FLAGS="-std=c++17 -O3 -fopenmp -DNDEBUG -w -I$REF -I$REF/third-party/eigen-3.4.0"
build_variant() {  # $1 = obj dir, $2 = extra defines
  local pids=()
  for s in $SRCS; do
    if [ ! -f "$1/$s.o" ] || [ "$REF/$s.cpp" -nt "$1/$s.o" ]; then
      g++ $FLAGS $2 -c "$REF/$s.cpp" -o "$1/$s.o" & pids+=($!)
    fi
  done
  for p in "${pids[@]}"; do wait "$p"; done
}
build_variant "$OUT/obj_real" ""
build_variant "$OUT/obj_cplx" "-DuseComplex"
g++ $FLAGS -I"$REF" "$HERE/ref_driver.cpp" "$OUT"/obj_real/*.o -o "$OUT/ref_driver" -lpthread
g++ $FLAGS -DuseComplex -I"$REF" "$HERE/ref_driver.cpp" "$OUT"/obj_cplx/*.o -o "$OUT/ref_driver_cplx" -lpthread
echo "built $OUT/ref_driver and $OUT/ref_driver_cplx"
