#!/bin/bash
# Compiles the reference's OWN callers of the engine, unmodified, against the
# GPU shim and libprothgpu.so, into oracle/_ref/ref_callers:
#
#   build_ref_callers.sh <prothlogic4.2 source directory>   (or PROTH_REF_SRC=<dir> ...)
#
# Reference files compiled as they are: dcore.cpp, worker.cpp, pipeline_proth.cpp,
# proth_logic.cpp, checkpoint_manager.cpp, storage_core.cpp, progress_core.cpp.
# fft_engine.cpp and llr_fft_pack.cpp are left out: the shim
# (prothlogic_gb300/compat/fft_engine_gpu.cpp, built with the reference's own
# fft_engine.h via -DPROTHGPU_USE_REFERENCE_HEADERS) provides fft_init,
# fft_square_karatsuba and fft_destroy.  GMP comes from the declaration-only
# header in gmpstub/ and the system libgmp.so.10.  Needs libprothgpu.so built
# first (python prothlogic_gb300/build.py) and a host that can compile both
# (no AVX-512 is needed: these files use none).
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REPO="$(cd "$HERE/../.." && pwd)"
SRC="${1:-$PROTH_REF_SRC}"
OUT="$HERE/../_ref"
LIBDIR="$REPO/prothlogic_gb300/_build"
[ -n "$SRC" ] || { echo "usage: build_ref_callers.sh <reference prothlogic4.2 directory>"; exit 1; }
[ -d "$SRC" ] || { echo "reference sources not found: $SRC"; exit 1; }
[ -f "$LIBDIR/libprothgpu.so" ] || { echo "build libprothgpu.so first"; exit 1; }
mkdir -p "$OUT"
FLAGS="-O2 -std=c++17 -pthread -w"
g++ $FLAGS -DPROTHGPU_USE_REFERENCE_HEADERS -I"$SRC" -c "$REPO/prothlogic_gb300/compat/fft_engine_gpu.cpp" \
    -o "$OUT/fft_engine_gpu_ref.o"
g++ $FLAGS -I"$HERE/gmpstub" -I"$SRC" -o "$OUT/ref_callers" "$HERE/ref_callers.cpp" \
    "$SRC/dcore.cpp" "$SRC/worker.cpp" "$SRC/pipeline_proth.cpp" "$SRC/proth_logic.cpp" \
    "$SRC/checkpoint_manager.cpp" "$SRC/storage_core.cpp" "$SRC/progress_core.cpp" \
    "$OUT/fft_engine_gpu_ref.o" -L"$LIBDIR" -lprothgpu -Wl,-rpath,"$LIBDIR" -l:libgmp.so.10
echo "built $OUT/ref_callers"
