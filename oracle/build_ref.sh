#!/usr/bin/env bash
# Builds the reference QMIV metric library from its own sources, in place where they
# lie, into oracle/_ref/ (git-ignored). Test infrastructure only: the outputs are the
# checker used to pin the C restatement in oracle/qmiv_oracle.c and to generate the
# golden fixtures under tests/golden/. Nothing in the product links or runs them.
#
# The reference's CMake build fetches fmt and doctest over the network, so this
# recipe compiles the translation units directly:
#   * fmt comes header-only from the copy shipped inside PyTorch's include tree;
#   * fmt 12 dropped fmt::localtime, used once by the CLI (apps/QMIV/src/xAppQMIV.cpp:975),
#     so a three-line stand-in is force-included (oracle/ref_fmt_localtime.h);
#   * libs/pmbb-ivqm/src/xIVPSNRM.cpp is skipped: it is not part of the library's
#     source list (libs/pmbb-ivqm/TargetSources.cmake:15-16) and includes a missing header.
# On x86-64 the build targets x86-64-v4 (the level the reference's runtime dispatcher
# picks on AVX-512 hosts); elsewhere it builds the portable STD code paths.
#
# Usage: oracle/build_ref.sh [REFERENCE_SOURCE_DIR]   (default $QMIV_REFERENCE_DIR, else /root/reference)
# Exits 3 without building when the sources are absent.
set -euo pipefail

HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
SRC="${1:-${QMIV_REFERENCE_DIR:-/root/reference}}"
# a machine without a reference checkout may carry the sources staged by oracle/stage_ref.sh
if [ ! -d "$SRC/libs/pmbb-ivqm/src" ] && [ -d "$HERE/../baseline/_ref/src/libs/pmbb-ivqm/src" ]; then
  SRC="$(cd "$HERE/../baseline/_ref/src" && pwd)"
fi
OUT="$HERE/_ref"
OBJ="$OUT/obj-$(uname -m)"

if [ ! -d "$SRC/libs/pmbb-ivqm/src" ]; then
  echo "reference sources not found at $SRC; skipping reference build" >&2
  exit 3
fi

FMT_INC="$(python3 -c 'import torch, os; print(os.path.join(os.path.dirname(torch.__file__), "include"))' 2>/dev/null || true)"
if [ -z "$FMT_INC" ] || [ ! -f "$FMT_INC/fmt/format.h" ]; then
  echo "fmt headers not found (looked in torch include dir)" >&2
  exit 4
fi

ARCH="$(uname -m)"
if [ "$ARCH" = "x86_64" ]; then MARCH="-march=x86-64-v4"; else MARCH=""; fi

mkdir -p "$OBJ"
CXXFLAGS=(-std=c++17 -O2 $MARCH -DFMT_HEADER_ONLY -w
          -I"$SRC/libs/pmbb-base/src" -I"$SRC/libs/pmbb-core/src" -I"$SRC/libs/pmbb-ivqm/src"
          -I"$SRC/libs/pmbb-spng/src" -I"$SRC/thirdparty/spng/src" -I"$FMT_INC"
          -include "$HERE/ref_fmt_localtime.h")

SOURCES=()
for f in "$SRC"/libs/pmbb-base/src/*.cpp "$SRC"/libs/pmbb-core/src/*.cpp "$SRC"/libs/pmbb-ivqm/src/*.cpp; do
  case "$(basename "$f")" in
    xIVPSNRM.cpp) continue ;;
    # processor identification by cpuid/xgetbv: x86 only; the metric library does not use it (the
    # command-line tool does, so on other hosts the tool does not link and qmiv_ref_timing stands in)
    xProcInfo.cpp) if [ "$ARCH" != "x86_64" ]; then continue; fi ;;
  esac
  SOURCES+=("$f")
done

pids=()
objs=()
for f in "${SOURCES[@]}"; do
  rel="${f#$SRC/}"
  o="$OBJ/$(echo "$rel" | tr '/' '_' ).o"
  objs+=("$o")
  if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then
    g++ "${CXXFLAGS[@]}" -c "$f" -o "$o" &
    pids+=($!)
    if [ "${#pids[@]}" -ge "$(nproc)" ]; then wait "${pids[0]}"; pids=("${pids[@]:1}"); fi
  fi
done
# the reference's own command-line tool (its published example values; the CPU baseline that
# bench.py times), compiled alongside
APP_OBJS=()
APP_SRCS=()
if [ "$ARCH" = "x86_64" ]; then APP_SRCS=("$SRC/apps/QMIV/src/main_QMIV.cpp" "$SRC/apps/QMIV/src/xAppQMIV.cpp" "$SRC"/libs/pmbb-spng/src/*.cpp); fi
for f in "${APP_SRCS[@]}"; do
  rel="${f#$SRC/}"
  o="$OBJ/$(echo "$rel" | tr '/' '_' ).o"
  if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then g++ "${CXXFLAGS[@]}" -c "$f" -o "$o" & pids+=($!); fi
  APP_OBJS+=("$o")
done
SPNG_SRCS=()
if [ "$ARCH" = "x86_64" ]; then SPNG_SRCS=("$SRC"/thirdparty/spng/src/spng.c "$SRC"/thirdparty/spng/src/miniz.c); fi
for f in "${SPNG_SRCS[@]}"; do
  o="$OBJ/$(basename "$f").o"
  if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then gcc -O2 -w -I"$SRC/thirdparty/spng/src" -c "$f" -o "$o" & pids+=($!); fi
  APP_OBJS+=("$o")
done
for p in "${pids[@]}"; do wait "$p"; done

# the checker harness and the checker of the input-side operations (colour conversion, range
# check / clipping): this repository's code, linked against the reference objects
g++ "${CXXFLAGS[@]}" "$HERE/ref_harness.cpp" "${objs[@]}" -lpthread -o "$OUT/qmiv_ref_harness" & l1=$!
g++ "${CXXFLAGS[@]}" "$HERE/ref_io.cpp" "${objs[@]}" -lpthread -o "$OUT/qmiv_ref_io" & l2=$!
# the timing driver of the CPU baseline (the application's per-frame steps around the library)
g++ "${CXXFLAGS[@]}" "$HERE/ref_timing.cpp" "${objs[@]}" -lpthread -o "$OUT/qmiv_ref_timing" & l3=$!
if [ "$ARCH" = "x86_64" ]; then
  g++ "${APP_OBJS[@]}" "${objs[@]}" -lpthread -o "$OUT/QMIV" || echo "note: reference CLI did not link; harness is still usable" >&2
fi
wait $l1
wait $l2
wait $l3

echo "reference build ready in $OUT"
