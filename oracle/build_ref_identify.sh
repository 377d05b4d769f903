#!/bin/sh
# Build the reference's identify application (targets/identify.cpp +
# src/hierarchy.cpp + src/HV.cpp + src/encoder.cpp of
# benlaflen/bacterial-classification, unmodified, compiled where they lie) for
# one compile-time configuration, with HVCache::precompute turned off inside
# identify.cpp by oracle/ref_identify_shim.h (compute-semantics windows).
# Output in oracle/_ref/.  Test infrastructure only; needs the reference.
#   sh oracle/build_ref_identify.sh <HV_DIM> <KMER_SIZE> <SEQUENCE_LENGTH> <SIM_STEP>
set -e
# the reference checkout: $REF_ROOT, else a directory "reference" beside this repository
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF_ROOT:-$(cd "$HERE/../.." && pwd)/reference}
D=$1; K=$2; L=$3; S=$4
[ -n "$S" ] || { echo "usage: $0 DIM KMER WINDOW STEP" >&2; exit 1; }
mkdir -p "$HERE/_ref"
OUT="$HERE/_ref/identify_D${D}_k${K}_L${L}_s${S}"
if [ -x "$OUT" ] && [ "$OUT" -nt "$HERE/ref_identify_shim.h" ]; then echo "$OUT"; exit 0; fi
TMP=$(mktemp -d)
FLAGS="-std=c++20 -O3 -march=native -ffast-math -DNORM_COSINE -DREF_HV_DIM=$D -DREF_KMER=$K -DREF_WINDOW=$L -DREF_STEP=$S"
INC="-include $REF/src/config.h -include $HERE/ref_config.h -I$REF/src"
for f in HV encoder hierarchy; do
    g++ $FLAGS $INC -c "$REF/src/$f.cpp" -o "$TMP/$f.o"
done
g++ $FLAGS $INC -include "$HERE/ref_identify_shim.h" -c "$REF/targets/identify.cpp" -o "$TMP/identify.o"
g++ "$TMP/identify.o" "$TMP/HV.o" "$TMP/encoder.o" "$TMP/hierarchy.o" -o "$OUT.tmp"
mv "$OUT.tmp" "$OUT"
rm -r "$TMP"
echo "$OUT"
