#!/bin/sh
# Builds oracle/_ref/libmbpol_ref.so: the MB-pol Reference-platform force
# classes compiled unmodified from the reference sources, plus the shim and
# the harness.  Needs the reference checkout: MBPOL_REFERENCE_DIR.
# The polynomial objects take minutes (poly-3b-v2x.cpp ~12 min at -O2) and
# are reused when present.  Outputs go to oracle/_ref only.
set -e
REF=${MBPOL_REFERENCE_DIR:?set MBPOL_REFERENCE_DIR to the reference checkout}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SRC="$REF/platforms/reference/src"
mkdir -p "$OUT"
INC="-I$HERE/shim -I$REF/openmmapi/include -I$REF/platforms/reference/include -I$SRC"
CXX=${CXX:-g++}
FLAGS="-O2 -fPIC -w"
pids=""
for f in MBPolReferenceOneBodyForce MBPolReferenceTwoBodyForce MBPolReferenceThreeBodyForce \
         ReferenceThreeNeighborList mbpol_2body_constants gammq MBPolReferenceElectrostaticsForce \
         poly-2b-v6x poly-3b-v2x; do
  if [ ! -f "$OUT/$f.o" ] || [ "$SRC/$f.cpp" -nt "$OUT/$f.o" ]; then
    $CXX $FLAGS $INC -c "$SRC/$f.cpp" -o "$OUT/$f.o" & pids="$pids $!"
  fi
done
$CXX $FLAGS $INC -c "$HERE/shim_fft.cpp" -o "$OUT/shim_fft.o" & pids="$pids $!"
$CXX $FLAGS $INC -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o" & pids="$pids $!"
$CXX $FLAGS $INC -c "$HERE/ref_poly.cpp" -o "$OUT/ref_poly2b.o" & pids="$pids $!"
$CXX $FLAGS $INC -DPOLY3B -c "$HERE/ref_poly.cpp" -o "$OUT/ref_poly3b.o" & pids="$pids $!"
for p in $pids; do wait $p; done
$CXX -shared -o "$OUT/libmbpol_ref.so" "$OUT"/*.o
echo "built $OUT/libmbpol_ref.so"
