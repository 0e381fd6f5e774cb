#!/usr/bin/env bash
# Build the reference's own CPU kernels (module `sscha_HP_odd`) from the C
# sources where they lie in the reference checkout, into oracle/_ref/.
# Test infrastructure only: the product never loads this module.
#   usage: oracle/build_ref.sh [REFERENCE_ROOT]
# (default $TDSCHA_REFERENCE_ROOT, else the directory "reference" beside this
# repository's checkout)
# Compiled from CModules/odd_corr_module.c + CModules/LanczosFunctions.c only;
# the prebuilt objects shipped next to them are never used. -O2 because the
# reference's Makefile notes a segfault at -O3 (CModules/Makefile:3).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${TDSCHA_REFERENCE_ROOT:-$(dirname "$(dirname "$HERE")")/reference}}"
OUT="$HERE/_ref"
if [ ! -f "$REF/CModules/LanczosFunctions.c" ]; then
  echo "reference sources not found under $REF; oracle/_ref not built" >&2
  exit 3
fi
mkdir -p "$OUT"
PYINC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
NPINC="$(python3 -c 'import numpy; print(numpy.get_include())')"
SUFFIX="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
gcc -O2 -fPIC -shared -fopenmp -w \
    -I"$PYINC" -I"$NPINC" -I"$REF/CModules" \
    "$REF/CModules/odd_corr_module.c" "$REF/CModules/LanczosFunctions.c" \
    -o "$OUT/sscha_HP_odd$SUFFIX" -lm
echo "built $OUT/sscha_HP_odd$SUFFIX"
