#!/usr/bin/env bash
# Test infrastructure only: builds the reference's own CPU driver (variants
# 'c' = fgls_chol and 'e' = fgls_eigen) from its unmodified C sources, for use
# as the parity checker and the timed CPU baseline.  Nothing here is part of
# the shipped library.
#
#   usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   (default: $FGLS_REFERENCE_ROOT, else DEFAULT_REF below)
#
# The reference links a Fortran-ABI BLAS/LAPACK (src/blas.h, src/lapack.h).
# This image has no system BLAS; scipy ships OpenBLAS with every symbol
# prefixed "scipy_".  We rename the undefined references in OUR objects with
# objcopy and link against that library.  Outputs go to oracle/_ref/ only.
set -euo pipefail
DEFAULT_REF=/root/reference
REF=${1:-${FGLS_REFERENCE_ROOT:-$DEFAULT_REF}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "build_ref: no reference sources at $REF/src; skipping" >&2
  exit 0
fi
OBLAS=$(python3 - << 'PY'
import glob, os, scipy
d = os.path.dirname(scipy.__file__)
c = sorted(glob.glob(os.path.join(d, "..", "scipy.libs", "libscipy_openblas*.so"))) + \
    sorted(glob.glob(os.path.join(d, ".libs", "libscipy_openblas*.so")))
print(os.path.realpath(c[0]) if c else "")
PY
)
if [ -z "$OBLAS" ]; then echo "build_ref: scipy OpenBLAS not found" >&2; exit 1; fi
mkdir -p "$OUT/obj"
SYMS="dgemm_ dcopy_ ddot_ dgemv_ dpotrf_ dpotri_ dscal_ dsyevr_ dsyrk_ dtrsm_ dtrsv_"
REDEF=""
for s in $SYMS; do REDEF="$REDEF --redefine-sym $s=scipy_$s"; done
OBJS=""
for f in common driver fgls_chol fgls_eigen io timing; do
  gcc -O2 -fopenmp -pthread -D_FILE_OFFSET_BITS=64 -w -I"$REF/src" \
      -c "$REF/src/$f.c" -o "$OUT/obj/$f.o"
  objcopy $REDEF "$OUT/obj/$f.o"
  OBJS="$OBJS $OUT/obj/$f.o"
done
gcc -fopenmp -pthread $OBJS "$OBLAS" -Wl,-rpath,"$(dirname "$OBLAS")" -lm -lrt -o "$OUT/driver.x"
echo "$OBLAS" > "$OUT/BLAS.txt"
echo "build_ref: built $OUT/driver.x against $OBLAS"
