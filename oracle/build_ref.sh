#!/usr/bin/env bash
# Builds the reference's own host move generator (sarona-RD/perft_gpu, read
# from its sources in place) into oracle/_ref/libperft_ref.so.
#
# TEST INFRASTRUCTURE ONLY: the result pins the oracle restatement and makes
# the golden vectors.  It needs the reference tree (REF_DIR, default
# /root/reference) and an x86-64 host: the reference's MoveGeneratorBitboard.h
# includes <x86intrin.h> on Linux, so this recipe does not build on Arm.
# Nothing is copied out of the reference tree; only the shim is ours.
# -O2 or higher is required: at -O0 the unused static hugeMemset in utils.h
# keeps a reference to cudaMemset.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF_DIR/MoveGeneratorBitboard.h" ]; then
    echo "build_ref: reference tree not found at $REF_DIR" >&2
    exit 3
fi
case "$(uname -m)" in
    x86_64|amd64) ;;
    *) echo "build_ref: reference host code needs x86intrin.h (x86-64 only)" >&2; exit 4 ;;
esac
mkdir -p "$OUT"
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
g++ -O3 -std=c++17 -fPIC -shared -w \
    -I"$REF_DIR" -I"$CUDA_INC" \
    "$HERE/ref_shim.cpp" \
    "$REF_DIR/GlobalVars.cpp" "$REF_DIR/Magics.cpp" "$REF_DIR/randoms.cpp" "$REF_DIR/util.cpp" \
    -o "$OUT/libperft_ref.so.tmp" -lpthread
mv "$OUT/libperft_ref.so.tmp" "$OUT/libperft_ref.so"
echo "build_ref: $OUT/libperft_ref.so"
