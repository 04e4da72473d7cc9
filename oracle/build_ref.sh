#!/usr/bin/env bash
# Builds the reference AnsatzEvolve library straight from its own sources, plus the
# pinning / timing driver oracle/ref_driver.cpp, into oracle/_ref/.  Test and
# measurement infrastructure only: oracle/_ref/ validates the C restatement in
# oracle/oracle.c, produces the golden fixtures under tests/golden/ and is the timed
# CPU baseline of bench.py.  The reference's CMake project needs gfortran, so the
# translation units are compiled directly.
#
#   oracle/build_ref.sh           real and complex variants (portable flags, for the
#                                 golden fixtures) -> ref_driver, ref_driver_cplx
#   oracle/build_ref.sh --stage   copy the sources this build reads (src/*.cpp, *.h,
#                                 Generated/, the vendored Eigen headers) into
#                                 oracle/_ref/src, so that a host without the checkout
#                                 (the aarch64 GPU host) can build the timing variant;
#                                 oracle/_ref/ is git-ignored: the copy is never committed
#   oracle/build_ref.sh --timing  the real variant as the reference's CMake project
#                                 builds it (-O3 plus native code generation: -march=native
#                                 on x86-64, -mcpu=native on aarch64, OpenMP, NDEBUG)
#                                 -> ref_driver_native
# Sources: AE_REFERENCE, else a `reference` checkout beside this repository, else the
# staged copy in oracle/_ref/src.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
REF=${AE_REFERENCE:-$HERE/../../reference}/src
[ -d "$REF" ] || REF=$OUT/src
[ -d "$REF" ] || { echo "reference sources not found (AE_REFERENCE, ../reference or oracle/_ref/src)" >&2; exit 2; }
SRCS="AnsatzManager AnsatzSynthInterface TUPSLoadingUtils ansatz benchmark csvwriter diis
      fusedevolve hamiltonianmatrix linalg logger operatorpool sparsematrix threadpool tupsquantities"
mode=${1:-all}

if [ "$mode" = "--stage" ]; then
    [ "$REF" != "$OUT/src" ] || { echo "nothing to stage from: no reference checkout" >&2; exit 2; }
    mkdir -p "$OUT/src/third-party/eigen-3.4.0"
    for s in $SRCS; do cp -p "$REF/$s.cpp" "$OUT/src/"; done
    cp -p "$REF"/*.h "$OUT/src/"
    cp -rp "$REF/Generated" "$OUT/src/"
    rm -rf "$OUT/src/third-party/eigen-3.4.0/Eigen"
    cp -rp "$REF/third-party/eigen-3.4.0/Eigen" "$OUT/src/third-party/eigen-3.4.0/"
    echo "staged the reference sources in $OUT/src"
    exit 0
fi

FLAGS="-std=c++17 -O3 -fopenmp -DNDEBUG -w -I$REF -I$REF/third-party/eigen-3.4.0"
build_variant() {  # $1 = obj dir, $2 = extra flags
    mkdir -p "$1"
    local pids=()
    for s in $SRCS; do
        if [ ! -f "$1/$s.o" ] || [ "$REF/$s.cpp" -nt "$1/$s.o" ]; then
            g++ $FLAGS $2 -c "$REF/$s.cpp" -o "$1/$s.o" & pids+=($!)
        fi
    done
    for p in "${pids[@]}"; do wait "$p"; done
}

if [ "$mode" = "--timing" ]; then
    case "$(uname -m)" in
        aarch64|arm64) NATIVE="-mcpu=native" ;;
        *) NATIVE="-march=native" ;;
    esac
    build_variant "$OUT/obj_native_$(uname -m)" "$NATIVE"
    g++ $FLAGS $NATIVE "$HERE/ref_driver.cpp" "$OUT/obj_native_$(uname -m)"/*.o -o "$OUT/ref_driver_native" -lpthread
    echo "built $OUT/ref_driver_native ($NATIVE)"
    exit 0
fi

build_variant "$OUT/obj_real" ""
build_variant "$OUT/obj_cplx" "-DuseComplex"
g++ $FLAGS "$HERE/ref_driver.cpp" "$OUT"/obj_real/*.o -o "$OUT/ref_driver" -lpthread
g++ $FLAGS -DuseComplex "$HERE/ref_driver.cpp" "$OUT"/obj_cplx/*.o -o "$OUT/ref_driver_cplx" -lpthread
echo "built $OUT/ref_driver and $OUT/ref_driver_cplx"
