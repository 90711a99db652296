#!/bin/sh
# Compile the reference's own CSR algorithm files, where they lie in the
# reference tree, against the stand-in headers in oracle/ref_shim/, into
# oracle/_ref/libref.so.  The reference tree is $ACCELGRAPH_REFERENCE, or a
# snapshot checked out beside this repository (../reference); where neither
# exists this script does nothing and the tests that need libref.so are
# skipped.  Test infrastructure only.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${ACCELGRAPH_REFERENCE:-$HERE/../../reference}"
OUT="$HERE/_ref"
SRC="$REF/02_capi_graph/src/algorithms/capi"
INC="$REF/02_capi_graph/include"
if [ ! -f "$SRC/pageRank.c" ]; then
    echo "build_ref.sh: reference sources not found under $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
CC="${CC:-gcc}"
FLAGS="-O2 -fPIC -std=gnu11 -ffp-contract=off -fopenmp -w"
INCS="-I$HERE/ref_shim -I$INC/config -I$INC/algorithms/capi -I$INC/capi_utils"
for f in pageRank BFS SPMV connectedComponents; do
    $CC $FLAGS $INCS -c "$SRC/$f.c" -o "$OUT/$f.o"
done
for f in ref_utils ref_capi_emu ref_harness; do
    $CC $FLAGS $INCS -c "$HERE/ref_shim/$f.c" -o "$OUT/$f.o"
done
$CC -shared -fopenmp -Wl,--no-undefined -o "$OUT/libref.so" \
    "$OUT/pageRank.o" "$OUT/BFS.o" "$OUT/SPMV.o" "$OUT/connectedComponents.o" \
    "$OUT/ref_utils.o" "$OUT/ref_capi_emu.o" "$OUT/ref_harness.o" -lm
rm -f "$OUT"/*.o
echo "built $OUT/libref.so"
