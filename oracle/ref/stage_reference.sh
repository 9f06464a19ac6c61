#!/bin/bash
# Stages the reference files that oracle/ref/Makefile compiles (unmodified)
# and that the tests read into the git-ignored reference-install folder
# baseline/_ref/cyrsoxs, so that a GPU machine (which has no copy of the
# reference) can build and run the reference.
#
#   oracle/ref/stage_reference.sh <reference source tree>
set -euo pipefail
if [ $# -ne 1 ]; then
  echo "usage: $0 <reference source tree>" >&2
  exit 2
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
REPO="$(cd "$HERE/../.." && pwd)"
SRC="$1"
DST="$REPO/baseline/_ref/cyrsoxs"
mkdir -p "$DST/src" "$DST/Data"
cp "$SRC/src/cudaMain.cu" "$SRC/src/RotationMatrix.cpp" "$SRC/src/pymain.cpp" "$DST/src/"
cp -r "$SRC/include" "$DST/"
cp "$SRC/Data/edgeSphereZYX.h5" "$SRC/Data/config.txt" "$SRC"/Data/Material*.txt "$DST/Data/"
cp "$SRC/LICENSE" "$DST/" 2>/dev/null || true
echo "staged reference files into $DST"
