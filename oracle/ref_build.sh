#!/bin/sh
# Builds the REFERENCE's own sources (LLNL Kripke, read in place, never copied) into oracle/_ref/:
#   oracle/_ref/libkripke_ref.so  the reference's generator, Kernel::* functions and solvers, plus
#                                 oracle/ref_driver.cpp (a C interface mirroring the oracle's)
#   oracle/_ref/kripke            the reference's own command-line driver (src/kripke.cpp)
# RAJA and camp are empty submodules in the reference tree, so the build uses the project-written
# stand-in in oracle/refshim/ (sequential loops, layouts, views).  No CMake, no MPI, no OpenMP.
# Test infrastructure only: it pins the oracle; the product never loads it.
#
#   sh oracle/ref_build.sh [reference-src-dir]     (default /root/reference/src)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
SRC=${1:-${KRIPKE_REF_SRC:-/root/reference/src}}
OUT="$HERE/_ref"
CXX=${CXX:-g++}
# -ffp-contract=off: two roundings per multiply-add, like the oracle (and an x86-64 build without -mfma)
FLAGS="-O2 -std=c++17 -ffp-contract=off -fPIC -w -I$HERE/refshim -I$SRC -I$HERE"
if [ ! -f "$SRC/Kripke/Kernel/LTimes.cpp" ]; then
  echo "ref_build: no reference sources under $SRC" >&2
  exit 2
fi
mkdir -p "$OUT/obj"
JOBS=$(nproc 2>/dev/null || echo 4)
( cd "$SRC" && find Kripke -name '*.cpp' && echo kripke.cpp ) | \
  xargs -P "$JOBS" -I{} sh -c 'o="$1/obj/$(echo "$2" | tr / _ | sed "s/\.cpp$/.o/")"; '"$CXX"' '"$FLAGS"' -c "$3/$2" -o "$o"' _ "$OUT" {} "$SRC"
$CXX $FLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/obj/ref_driver.o"
LIBOBJS=$(ls "$OUT"/obj/*.o | grep -v '/kripke\.o$')
$CXX -shared -o "$OUT/libkripke_ref.so" $LIBOBJS
$CXX -o "$OUT/kripke" $(ls "$OUT"/obj/*.o | grep -v '/ref_driver\.o$')
echo "ref_build: $OUT/libkripke_ref.so $OUT/kripke"
