#!/bin/bash
# Builds the UNMODIFIED reference engine + ref_harness.cpp into oracle/_ref/.
#
#   build_ref.sh <prothlogic4.2 source directory>     (or PROTH_REF_SRC=<dir> build_ref.sh)
#
# Needs the reference sources and an x86-64 host with AVX-512 (the reference
# engine uses AVX-512 intrinsics and x86 inline assembly).
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
SRC="${1:-$PROTH_REF_SRC}"
OUT="$HERE/../_ref"
[ -n "$SRC" ] || { echo "usage: build_ref.sh <reference prothlogic4.2 directory>"; exit 1; }
[ -d "$SRC" ] || { echo "reference sources not found: $SRC"; exit 1; }
[ "$(uname -m)" = "x86_64" ] || { echo "reference needs x86-64 (AVX-512)"; exit 1; }
mkdir -p "$OUT"
# SETUP:25 flags, without -lgmpxx/-lcufft (unused on this path)
FLAGS="-O3 -march=native -mavx512f -mfma -funroll-loops -fomit-frame-pointer -mprefer-vector-width=512 -ffast-math -std=c++17 -pthread"
g++ $FLAGS -I"$HERE/gmpstub" -I"$SRC" -o "$OUT/ref_harness" \
    "$HERE/ref_harness.cpp" "$SRC/fft_engine.cpp" "$SRC/llr_fft_pack.cpp" "$SRC/checkpoint_manager.cpp" \
    "$SRC/proth_logic.cpp" "$SRC/storage_core.cpp" -l:libgmp.so.10 -w
echo "built $OUT/ref_harness"
