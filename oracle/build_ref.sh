#!/bin/bash
# build_ref.sh -- compiles the reference's own kernel sources for the CPU into oracle/_ref/libref_kernels.so.
#
# TEST INFRASTRUCTURE: the result pins the CPU oracle (oracle/lfrv_oracle.cpp) against the reference's
# kernels, bit for bit where both evaluate the same float operations (tests/test_oracle_ref.py). It is built
# only on a machine that has the reference tree; nothing is copied into the repository: the generated
# translation units under oracle/_ref/ (git-ignored) #include the reference files where they lie, or
# extract line ranges of files that also contain host-side launch code.
#
# usage: oracle/build_ref.sh [<reference root>]    (default: $LFRV_REFERENCE_ROOT, else /root/reference)
#        oracle/build_ref.sh --probe               (exit 0 and print the root if a reference tree is there)
set -euo pipefail
if [ "${1:-}" = "--probe" ]; then
    ROOT_DIR="${LFRV_REFERENCE_ROOT:-/root/reference}"
    [ -f "$ROOT_DIR/sources/optimization.cu" ] || exit 1
    echo "$ROOT_DIR"
    exit 0
fi
REF="${1:-${LFRV_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
mkdir -p "$OUT"

SR="$REF/cocolib/cocolib/vtv/vtv_sr_kernels_unstructured.cu"
ROF="$REF/cocolib/cocolib/vtv/vtv_rof.cu"
KER="$REF/cocolib/cocolib/cuda/cuda_kernels.cu"
SRK="$REF/cocolib/cocolib/vtv/vtv_sr_kernels.cu"
GRAD="$REF/sources/gradientIBR_kernels.cuh"
OPT="$REF/sources/optimization.cu"

# extract <file> <first> <last> <expected symbol> <out>
extract() {
    sed -n "$2,$3p" "$1" > "$5"
    if ! grep -q "$4" "$5"; then
        echo "build_ref.sh: $1:$2-$3 does not contain $4 (reference changed?)" >&2
        exit 1
    fi
}
extract "$ROF" 28 45 coco_vtv_rof_overrelaxation_device "$OUT/rof_overrelax.inc"
extract "$ROF" 118 147 coco_vtv_rof_dual_step_device "$OUT/rof_dual.inc"
extract "$ROF" 280 321 coco_vtv_rof_reproject_3D_tvf_weighted_device "$OUT/rof_reproject.inc"
extract "$KER" 79 339 cuda_normalize_device "$OUT/elementwise.inc"
extract "$KER" 504 533 cuda_rof_primal_prox_step_device "$OUT/primal_prox.inc"
extract "$SRK" 1172 1195 vtv_sr_init_regularizer_weight_device "$OUT/regweight.inc"
extract "$OPT" 210 542 "void expand" "$OUT/pushpull.inc"

cat > "$OUT/ref_sr.cpp" <<EOF
#include "$HERE/ref_shim.h"
#include "$SR"
#include "$OUT/rof_overrelax.inc"
#include "$OUT/rof_dual.inc"
#include "$OUT/rof_reproject.inc"
#include "$OUT/elementwise.inc"
#include "$OUT/primal_prox.inc"
#include "$OUT/regweight.inc"
#include "$HERE/ref_wrap_sr.inc"
EOF
cat > "$OUT/ref_grad.cpp" <<EOF
#include "$HERE/ref_shim.h"
#include "$GRAD"
#include "$HERE/ref_wrap_grad.inc"
EOF
cat > "$OUT/ref_pp.cpp" <<EOF
#include "$HERE/ref_shim.h"
#include "$OUT/pushpull.inc"
#include "$HERE/ref_wrap_pp.inc"
EOF

CXXFLAGS="-std=c++17 -O1 -fPIC -ffp-contract=off -w"
g++ $CXXFLAGS -c "$OUT/ref_sr.cpp" -o "$OUT/ref_sr.o"
g++ $CXXFLAGS -c "$OUT/ref_grad.cpp" -o "$OUT/ref_grad.o"
g++ $CXXFLAGS -c "$OUT/ref_pp.cpp" -o "$OUT/ref_pp.o"
g++ -shared -o "$OUT/libref_kernels.so" "$OUT/ref_sr.o" "$OUT/ref_grad.o" "$OUT/ref_pp.o"
echo "built $OUT/libref_kernels.so"
