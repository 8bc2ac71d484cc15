#!/bin/sh
# Compile the reference's own hot-path sources, read in place from the
# reference checkout (never copied), together with oracle/ref_harness.cpp and
# the single-rank MPI stand-in, into oracle/_ref/:
#   libasmooth_ref.so      serial, -ffp-contract=off  (parity: bit-exact outputs)
#   libasmooth_ref_omp.so  same with -fopenmp          (timing only)
# Usage: oracle/build_ref.sh <reference_dir>   (or $ASMOOTH_REFERENCE)
# Exits 0 without building when no directory is given or it holds no reference.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${ASMOOTH_REFERENCE:-}}
if [ -z "$REF" ]; then
    echo "build_ref: no reference directory given (argument or ASMOOTH_REFERENCE); nothing built"
    exit 0
fi
if [ ! -f "$REF/nbr_search.cpp" ]; then
    echo "build_ref: reference sources not found at $REF; nothing built"
    exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
SRCS=""
for f in nbr_search.cpp kdtree_balanced.cpp coarse_mesh.cpp fof.cpp basic_types.cpp \
         open.cpp global_mesh.cpp mpi_interface.cpp exchange_buffer.cpp file_reader2.cpp; do
    SRCS="$SRCS $REF/$f"
done
# -iquote: the reference's endian.h must not shadow the system <endian.h>
FLAGS="-O2 -ffp-contract=off -fPIC -shared -w -iquote $REF -I$HERE/mpi_shim"
g++ $FLAGS -o "$OUT/libasmooth_ref.so" "$HERE/ref_harness.cpp" $SRCS &
g++ $FLAGS -fopenmp -o "$OUT/libasmooth_ref_omp.so" "$HERE/ref_harness.cpp" $SRCS &
wait
echo "build_ref: built $OUT/libasmooth_ref.so $OUT/libasmooth_ref_omp.so"
