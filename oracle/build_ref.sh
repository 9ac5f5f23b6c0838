#!/usr/bin/env bash
# Builds the reference libffrs pybind11 extension from its own sources into
# oracle/_ref/ so that the C restatement in oracle/ can be checked against it
# and so that tests/golden/make_golden.py can generate fixtures.
#
# This is test infrastructure only: nothing in the libffrs_gb300 product path
# loads oracle/_ref.  The reference sources are read where they lie; nothing is
# copied into this repository.  The recipe mirrors the reference's own
# CMakeLists.txt (per-TU ISA flags, C++20, -O3) without running cmake.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
set -euo pipefail

REF=${1:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$REF/libffrs"

if [ ! -f "$SRC/pyffrs.cpp" ]; then
    echo "reference sources not found under $REF" >&2
    exit 2
fi

PYBIND_INC="$(python3 -c 'import pybind11; print(pybind11.get_include())' 2>/dev/null || true)"
if [ -z "$PYBIND_INC" ]; then
    # torch ships the pybind11 headers as well
    PYBIND_INC="$(python3 -c 'import torch, os; print(os.path.join(os.path.dirname(torch.__file__), "include"))')"
fi
PY_INC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
SUF="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"

mkdir -p "$OUT/obj"
CXX=${CXX:-g++}
FLAGS=(-O3 -std=c++20 -fPIC -I"$PYBIND_INC" -I"$PY_INC" -I"$SRC" -DVERSION_INFO='"ref-oracle"' -w)

ARCH="$(uname -m)"
objs=()
if [ "$ARCH" = "x86_64" ]; then
    "$CXX" "${FLAGS[@]}" -c "$SRC/pyffrs.cpp" -o "$OUT/obj/pyffrs.o" &
    "$CXX" "${FLAGS[@]}" -c "$SRC/rsi16v.cpp" -o "$OUT/obj/rsi16v.o" &
    "$CXX" "${FLAGS[@]}" -msse -msse2 -c "$SRC/rsi16v_sse2.cpp" -o "$OUT/obj/rsi16v_sse2.o" &
    "$CXX" "${FLAGS[@]}" -mavx2 -c "$SRC/rsi16v_avx2.cpp" -o "$OUT/obj/rsi16v_avx2.o" &
    "$CXX" "${FLAGS[@]}" -mavx512f -mavx512dq -c "$SRC/rsi16v_avx512.cpp" -o "$OUT/obj/rsi16v_avx512.o" &
    wait
    objs=("$OUT"/obj/pyffrs.o "$OUT"/obj/rsi16v.o "$OUT"/obj/rsi16v_sse2.o "$OUT"/obj/rsi16v_avx2.o "$OUT"/obj/rsi16v_avx512.o)
else
    echo "x86 SIMD translation units of the reference do not build on $ARCH" >&2
    exit 3
fi

"$CXX" -shared -o "$OUT/libffrs$SUF" "${objs[@]}"
echo "built $OUT/libffrs$SUF"
