#!/bin/bash
# Test infrastructure: builds the reference (dronperminov/FlipGraphGPU) from its
# own sources so that it can serve as the oracle's oracle on the GPU machine.
#
#  1. When the reference tree is present (FG_REFERENCE_DIR, default
#     /root/reference), its src/ is staged twice under oracle/_ref/:
#       src_zt  verbatim (the reference's default ring: SCHEME_INTEGER, "ZT")
#       src_z2  verbatim except that the ring switch at config.cuh:6 is
#               commented out, which is how the reference selects Z2.
#     The staged copies are build inputs only; oracle/_ref/ is git-ignored.
#  2. When nvcc is present, both variants are compiled with oracle/ref.mk
#     (the reference's own flags plus -gencode for sm_103a and the
#     `-include cstdint` shim its config.cuh needs) into
#     oracle/_ref/{zt,z2}-<machine> (x86_64 here, aarch64 on the GPU machine).
#     `build_ref.sh harness` builds only ref_harness (what the benchmark's
#     reference-CUDA leg runs); no argument builds the three executables too.
#
# Nothing here modifies the reference tree, and nothing in the product links or
# executes the result: it is used to generate and re-check tests/golden/, and
# bench.py runs ref_harness beside the product as the reference-CUDA baseline.
set -e
cd "$(dirname "$0")/.."
REF="${FG_REFERENCE_DIR:-/root/reference}"
OUT=oracle/_ref
mkdir -p "$OUT"
if [ -d "$REF/src" ]; then
    rm -rf "$OUT/src_zt" "$OUT/src_z2"
    cp -r "$REF/src" "$OUT/src_zt"
    cp -r "$REF/src" "$OUT/src_z2"
    sed -i 's|^#define SCHEME_INTEGER|// #define SCHEME_INTEGER|' "$OUT/src_z2/config.cuh"
fi
if [ ! -d "$OUT/src_zt" ]; then
    echo "build_ref: no staged reference sources; skipping" >&2
    exit 0
fi
if ! command -v nvcc >/dev/null 2>&1; then
    echo "build_ref: nvcc not found; skipping" >&2
    exit 0
fi
JOBS="${FG_JOBS:-$(nproc)}"
ARCHDIR="$(uname -m)"
TZT=""; TZ2=""
if [ "${1:-}" = "harness" ]; then TZT="$OUT/zt-$ARCHDIR/ref_harness"; TZ2="$OUT/z2-$ARCHDIR/ref_harness"; fi
make -s -j"$JOBS" -f oracle/ref.mk SRC="$OUT/src_zt" OUT="$OUT/zt-$ARCHDIR" $TZT &
P1=$!
make -s -j"$JOBS" -f oracle/ref.mk SRC="$OUT/src_z2" OUT="$OUT/z2-$ARCHDIR" $TZ2 &
P2=$!
wait $P1; R1=$?
wait $P2; R2=$?
exit $(( R1 | R2 ))
