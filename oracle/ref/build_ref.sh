#!/usr/bin/env bash
# Builds the reference library's hot path for the CPU, once per moduli set, from
# the unmodified headers under the reference checkout:
#   oracle/_ref/libmpres_ref_<N>.so   (N = 8, 16, 32 moduli of 32 bits)
# and its device code for the GB300, with the constants it computes at start-up:
#   oracle/_ref/ref_kernels_<N>.cubin, oracle/_ref/ref_consts_<N>.bin
# Needs the reference sources (REF_SRC, default /root/reference/src) and the
# GMP/MPFR runtime libraries; the headers for those come from oracle/ref/shim.
# Test infrastructure only: the output pins the oracle and makes golden vectors.
# This recipe is the one place that names the checkout's location:
#   build_ref.sh --where   prints the checkout root and exits 0, or exits 1 when
#                          the sources are absent (the GPU machine has none).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ORACLE="$(dirname "$HERE")"
REF_SRC="${REF_SRC:-/root/reference/src}"
OUT="$ORACLE/_ref"
if [ "${1:-}" = "--where" ]; then
    if [ -d "$REF_SRC" ]; then dirname "$REF_SRC"; exit 0; fi
    exit 1
fi
if [ ! -d "$REF_SRC" ]; then
    echo "reference sources not found at $REF_SRC; skipping oracle/_ref" >&2
    exit 0
fi
find_lib() {
    for d in /usr/lib/x86_64-linux-gnu /usr/lib/aarch64-linux-gnu /usr/lib64 /usr/lib; do
        if [ -e "$d/$1" ]; then echo "$d/$1"; return 0; fi
    done
    return 1
}
GMP="$(find_lib libgmp.so.10)" || { echo "libgmp.so.10 not found; skipping" >&2; exit 0; }
MPFR="$(find_lib libmpfr.so.6)" || { echo "libmpfr.so.6 not found; skipping" >&2; exit 0; }
mkdir -p "$OUT"
pids=()
for N in ${REF_SETS:-8 16 32}; do
    PARAMS="$REF_SRC/params/32-bit-moduli/params.${N}_32bit.h"
    g++ -std=c++17 -O2 -fPIC -shared -w \
        -frounding-math -fno-fast-math -ffp-contract=off \
        -I"$REF_SRC" -I"$HERE/shim" -I"$HERE" -I"$ORACLE" \
        -include "$PARAMS" \
        "$HERE/ref_harness.cpp" -o "$OUT/libmpres_ref_${N}.so" \
        "$MPFR" "$GMP" &
    pids+=($!)
done
# the reference's device code as a cubin for the GB300 (oracle/ref/gpu_harness.cu)
NVCC="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
if [ -x "$NVCC" ]; then
    for N in ${REF_SETS:-8 16 32}; do
        PARAMS="$REF_SRC/params/32-bit-moduli/params.${N}_32bit.h"
        "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -w \
            -I"$REF_SRC" -I"$HERE/shim" -include "$PARAMS" \
            "$HERE/gpu_harness.cu" -o "$OUT/ref_kernels_${N}.cubin" &
        pids+=($!)
    done
fi
for p in "${pids[@]}"; do wait "$p"; done
# the device constants the reference computes at start-up, for the cubin
python3 "$HERE/dump_consts.py" ${REF_SETS:-8 16 32} > /dev/null
echo "built $(ls "$OUT"/libmpres_ref_*.so | wc -l) reference libraries in $OUT"
