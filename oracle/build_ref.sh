#!/usr/bin/env bash
# Builds the UNMODIFIED reference DM-QR C sources (mdessole/qrdm, src/*.c) into
# oracle/_ref/libqrdm_ref.so so that the oracle and the GPU path can be pinned
# against the reference itself.  Test infrastructure only: nothing in the
# product links or loads this library.
#
# The reference links a system LAPACK/LAPACKE/CBLAS (setup_QRDM.py:13-17).  None
# is installed here, so the BLAS/LAPACK provider is the OpenBLAS bundled with
# scipy, whose symbols carry a `scipy_` prefix; a generated header maps the
# reference's unprefixed names onto them.  Sources are compiled where they lie
# (read-only), outputs go to oracle/_ref/ only.
#
# Usage: oracle/build_ref.sh <reference_root>   (or QRDM_REFERENCE_ROOT in the environment)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${QRDM_REFERENCE_ROOT:-}}"
if [ -z "$REF" ]; then
  echo "build_ref: no reference root given (argument or QRDM_REFERENCE_ROOT); skipping" >&2
  exit 0
fi
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "build_ref: reference sources not found at $REF; skipping" >&2
  exit 0
fi
OPENBLAS="$(python3 -c 'import scipy,os,glob; print(sorted(glob.glob(os.path.dirname(scipy.__file__)+".libs/libscipy_openblas*.so"))[0])')"
mkdir -p "$OUT"
SHIM="$OUT/shim.h"
{
  echo "/* generated by oracle/build_ref.sh: map LAPACKE/CBLAS names to scipy-openblas */"
  for s in LAPACKE_dge_nancheck LAPACKE_dgeqp3 LAPACKE_dgeqp3_work LAPACKE_dgeqpf \
           LAPACKE_dgeqrf LAPACKE_dlamch LAPACKE_dlarfb_work LAPACKE_dlarft \
           LAPACKE_dormqr LAPACKE_dtr_nancheck LAPACKE_get_nancheck LAPACKE_lsame \
           LAPACKE_xerbla cblas_dgemv cblas_dger cblas_dnrm2 cblas_dscal cblas_dswap \
           cblas_dsyrk dlapy2_ iladlc_ iladlr_ xerbla_; do
    echo "#define $s scipy_$s"
  done
} > "$SHIM"
SRCS=""
for f in dlarfb dlarf dlarfg dgeqr2 dgeqp3 dgeqrdm_work dgeqrdm; do SRCS="$SRCS $REF/src/$f.c"; done
# -O2 is required: at -O0 the dead tail of dgeqrdm_work (apply_jpvt, DM_perm2)
# leaves undefined symbols in the shared object.
gcc -O2 -fPIC -shared -include "$SHIM" -I"$REF/include" -w $SRCS \
    "$OPENBLAS" -Wl,-rpath,"$(dirname "$OPENBLAS")" -lm -o "$OUT/libqrdm_ref.so"
echo "$OPENBLAS" > "$OUT/openblas_path.txt"
echo "build_ref: built $OUT/libqrdm_ref.so against $OPENBLAS"
