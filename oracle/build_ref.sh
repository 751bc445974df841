#!/usr/bin/env bash
# Builds the reference's own host move generator (sarona-RD/perft_gpu, read
# from its sources in place) into oracle/_ref/libperft_ref.so.
#
# TEST INFRASTRUCTURE ONLY: the result pins the oracle restatement and makes
# the golden vectors.  It needs the reference tree: REF_DIR, default the
# directory "reference" beside this repository.  The reference's
# MoveGeneratorBitboard.h includes <x86intrin.h> on Linux for _mm_popcnt_u64;
# on a host that is not x86-64 (or with REF_SHIM=1) arm_include/ goes first
# on the include path, whose x86intrin.h defines that intrinsic over
# __builtin_popcountll.  The reference files are compiled unchanged and read
# in place; nothing is copied out of the reference tree; only the shims are
# ours.
# -fsigned-char keeps x86-64 semantics for plain char on aarch64.
# -O2 or higher is required: at -O0 the unused static hugeMemset in utils.h
# keeps a reference to cudaMemset.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:-$HERE/../../reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF_DIR/MoveGeneratorBitboard.h" ]; then
    echo "build_ref: reference tree not found at $REF_DIR" >&2
    exit 3
fi
SHIM_INC=()
case "$(uname -m)" in
    x86_64|amd64) [ "${REF_SHIM:-0}" = 1 ] && SHIM_INC=(-I"$HERE/arm_include") ;;
    *) SHIM_INC=(-I"$HERE/arm_include") ;;
esac
mkdir -p "$OUT"
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
g++ -O3 -std=c++17 -fPIC -shared -w -fsigned-char \
    "${SHIM_INC[@]}" -I"$REF_DIR" -I"$CUDA_INC" \
    "$HERE/ref_shim.cpp" \
    "$REF_DIR/GlobalVars.cpp" "$REF_DIR/Magics.cpp" "$REF_DIR/randoms.cpp" "$REF_DIR/util.cpp" \
    -o "$OUT/libperft_ref.so.tmp" -lpthread
mv "$OUT/libperft_ref.so.tmp" "$OUT/libperft_ref.so"
echo "build_ref: $OUT/libperft_ref.so"
