#!/bin/bash
# Stages the reference sources that oracle/ref/Makefile compiles (unmodified)
# into the git-ignored reference-install folder baseline/_ref/cyrsoxs, so that
# a GPU machine (which has no /root/reference) can build and run the reference to
# produce golden vectors.  Run in the development container only.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REPO="$(cd "$HERE/../.." && pwd)"
SRC="${1:-/root/reference}"
DST="$REPO/baseline/_ref/cyrsoxs"
mkdir -p "$DST/src"
cp "$SRC/src/cudaMain.cu" "$SRC/src/RotationMatrix.cpp" "$DST/src/"
cp -r "$SRC/include" "$DST/"
cp "$SRC/LICENSE" "$DST/" 2>/dev/null || true
echo "staged reference sources into $DST"
