#!/bin/sh
# Compiles the reference's own src/core.cpp (unmodified, read where it lies) into
# oracle/_ref/libref_core.so, with the shim MKL header and plain-loop cblas of
# oracle/shim.  Test infrastructure: the checker for oracle.c.  The reference checkout is
# named by the first argument or $SPTRSV_REFERENCE; with neither, or when the directory holds
# no src/core.cpp (a host without a reference checkout), it exits 0 without building.  The reference's utils.cpp is
# not built: it includes <c++/7/bits/c++config.h> (utils.cpp:3), which gcc 13 lacks.
set -e
REF="${1:-${SPTRSV_REFERENCE:-}}"
if [ -z "$REF" ]; then echo "build_ref: no reference checkout named (argument or SPTRSV_REFERENCE), skipped"; exit 0; fi
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$REF/src/core.cpp" ]; then echo "build_ref: no reference at $REF, skipped"; exit 0; fi
mkdir -p "$HERE/_ref"
gcc -O2 -fPIC -c "$HERE/shim/cblas_naive.c" -I"$HERE/shim" -o "$HERE/_ref/cblas_naive.o"
g++ -O2 -fPIC -fopenmp -w -c "$REF/src/core.cpp" -I"$REF" -I"$HERE/shim" -o "$HERE/_ref/core.o"
g++ -O2 -fPIC -c "$HERE/shim/ref_wrap.cpp" -o "$HERE/_ref/ref_wrap.o"
g++ -shared -fopenmp -Wl,-Bsymbolic -o "$HERE/_ref/libref_core.so" \
    "$HERE/_ref/core.o" "$HERE/_ref/ref_wrap.o" "$HERE/_ref/cblas_naive.o"
echo "build_ref: built $HERE/_ref/libref_core.so"
