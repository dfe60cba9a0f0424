#!/usr/bin/env bash
# ORACLE TEST INFRASTRUCTURE — not part of the product.
#
# Compiles the UNMODIFIED reference GCGE core (src/*.c) and its CSR app
# (app/csr/gcge_app_csr.c) from the read-only reference checkout, together
# with oracle/ref_driver.c and oracle/ref_blas_shim.c, into
# oracle/_ref/libgcge_ref.so.  No reference source is copied: gcc reads the
# files where they lie.  The reference's gcge_config.h switches MPI on; its
# include guard is pre-defined here and the same four macros are given on the
# command line with MPI off (what the reference Makefile does with sed,
# Makefile:34-38).  LAPACK/BLAS come from scipy's bundled OpenBLAS.
#
# Usage: oracle/build_ref.sh REFERENCE_DIR   (or GCGE_REFERENCE_DIR set)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${GCGE_REFERENCE_DIR:-}}"
if [ -z "$REF" ]; then
  echo "usage: $0 REFERENCE_DIR (or set GCGE_REFERENCE_DIR)" >&2
  exit 2
fi
OUT="$HERE/_ref"
if [ ! -f "$REF/src/gcge_eigsol.c" ]; then
  echo "reference sources not found under $REF; oracle/_ref not built" >&2
  exit 2
fi
BLASDIR="$(python3 -c 'import scipy, os; print(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs"))')"
BLASLIB="$(ls "$BLASDIR" | grep -E '^libscipy_openblas.*\.so' | head -1)"
if [ -z "$BLASLIB" ]; then
  echo "scipy OpenBLAS not found in $BLASDIR" >&2
  exit 3
fi
mkdir -p "$OUT"
gcc -O2 -fPIC -shared -w \
  -D_GCGE_CONFIG_H_ -DGCGE_DOUBLE=double -DGCGE_INT=int -DGET_PART_TIME=1 -DGCGE_USE_MPI=0 \
  -include float.h \
  -I"$REF/src" -I"$REF/app/csr" \
  "$REF"/src/gcge_*.c "$REF/app/csr/gcge_app_csr.c" \
  "$HERE/ref_driver.c" "$HERE/ref_blas_shim.c" \
  -L"$BLASDIR" -l:"$BLASLIB" -Wl,-rpath,"$(cd "$BLASDIR" && pwd)" -lm \
  -o "$OUT/libgcge_ref.so"
echo "built $OUT/libgcge_ref.so"
