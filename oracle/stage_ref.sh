#!/usr/bin/env bash
# Stages the reference's sources that oracle/build_ref.sh compiles (libs/pmbb-{base,core,ivqm,spng},
# apps/QMIV, thirdparty/spng) into baseline/_ref/src/, which git ignores: they are never committed,
# but they travel with the working tree to a machine that has no reference checkout, where
# oracle/build_ref.sh builds the reference's own metric library and command-line tool for that
# machine's architecture (the portable code paths on aarch64). The built tool is the CPU baseline
# that bench.py times beside the GPU numbers. Test infrastructure only.
#
# Usage: oracle/stage_ref.sh [REFERENCE_SOURCE_DIR]   (default $QMIV_REFERENCE_DIR, else /root/reference)
set -euo pipefail

HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
SRC="${1:-${QMIV_REFERENCE_DIR:-/root/reference}}"
DST="$HERE/../baseline/_ref/src"

if [ ! -d "$SRC/libs/pmbb-ivqm/src" ]; then
  echo "reference sources not found at $SRC" >&2
  exit 3
fi
for d in libs/pmbb-base/src libs/pmbb-core/src libs/pmbb-ivqm/src libs/pmbb-spng/src apps/QMIV/src thirdparty/spng/src; do
  mkdir -p "$DST/$d"
  cp -p "$SRC/$d"/*.h "$SRC/$d"/*.c* "$DST/$d"/ 2>/dev/null || true
done
cp -p "$SRC/LICENSE" "$DST/" 2>/dev/null || true
echo "staged reference sources in $(cd "$DST" && pwd)"
