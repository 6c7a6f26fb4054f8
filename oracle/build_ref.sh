#!/usr/bin/env bash
# Builds the reference's own CPU program as a checker, from its sources where
# they lie (read-only), into oracle/_ref/.  Nothing is copied into the repo.
#
#   oracle/_ref/uvatrmm.x    the unmodified reference program (uvatrmm.x), one rank
#   oracle/_ref/ref_harness  oracle/ref_harness.c linked with the reference's
#                            mapping and data-generation code
#
# Flags follow UVaTRMM/Makefile:13-14 (-O3 -fopenmp -std=c99 -DMININUMS=1).
# MPI is replaced by the single-rank stub oracle/shim/mpi.h and MKL by
# oracle/shim/mkl.h over the OpenBLAS that scipy bundles.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# REFERENCE_ROOT is the argument, else $UVATRMM_REFERENCE_ROOT, else a
# checkout named `reference` beside this repository's directory.  Exits 0 and
# builds nothing when the reference tree is absent.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${UVATRMM_REFERENCE_ROOT:-$HERE/../../reference}}"
SRC="$REF/UVaTRMM"
if [ ! -d "$SRC/src" ]; then
  echo "build_ref: reference sources not found at $SRC; skipping" >&2
  exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
BLAS="$(python3 - <<'EOF'
import glob, os, scipy
c = sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__), '..', 'scipy.libs', 'libscipy_openblas*.so')))
print(os.path.realpath(c[0]) if c else '')
EOF
)"
if [ -z "$BLAS" ]; then echo "build_ref: scipy OpenBLAS not found" >&2; exit 1; fi
BLASDIR="$(dirname "$BLAS")"
CFLAGS="-O3 -fopenmp -std=c99 -DMININUMS=1 -w -I$HERE/shim -I$SRC -I$SRC/include -I$SRC/src"
LIBS="$BLAS -Wl,-rpath,$BLASDIR -lm"
gcc $CFLAGS "$SRC/src/mm_triangular.c" "$SRC/src/mm_triangular_common.c" "$SRC/src/mm_mapping.c" \
    "$SRC/src/mm_comm_split.c" $LIBS -o "$OUT/uvatrmm.x"
gcc $CFLAGS "$HERE/ref_harness.c" "$SRC/src/mm_triangular_common.c" "$SRC/src/mm_mapping.c" \
    "$SRC/src/mm_comm_split.c" $LIBS -o "$OUT/ref_harness"
echo "build_ref: built $OUT/uvatrmm.x and $OUT/ref_harness against $BLAS"
