#!/bin/sh
# Builds the reference's MolEmb extension from its own source tree into
# oracle/_ref/ (git-ignored). Needs the reference tree at $TM_REFERENCE, or
# else in a `reference` directory beside the repository checkout; where it is
# absent the script exits 0 and prints why, and the oracle restatement is used
# alone.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${TM_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}"
SRC="$REF/C_API/MolEmb.cpp"
if [ ! -f "$SRC" ]; then
  echo "build_ref: reference source not present ($SRC); skipping"
  exit 0
fi
mkdir -p "$HERE/_ref"
PY="${PYTHON:-python3}"
PYINC=$($PY -c "import sysconfig;print(sysconfig.get_paths()['include'])")
NPINC=$($PY -c "import numpy;print(numpy.get_include())")
SUF=$($PY -c "import sysconfig;print(sysconfig.get_config_var('EXT_SUFFIX'))")
OUT="$HERE/_ref/MolEmb$SUF"
if [ -f "$OUT" ] && [ "$OUT" -nt "$SRC" ]; then
  exit 0
fi
# setup.py:15-20 of the reference builds with -std=c++0x -fopenmp
g++ -O2 -shared -fPIC -std=c++0x -fopenmp -w -include "$HERE/molemb_compat.h" \
    -I"$PYINC" -I"$NPINC" -I"$REF/C_API" "$SRC" -o "$OUT"
echo "build_ref: built $OUT"
