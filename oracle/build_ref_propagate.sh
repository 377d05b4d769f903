#!/bin/sh
# Build the reference's propagate-children application
# (targets/propogate-children.cpp + src/hierarchy.cpp + src/HV.cpp +
# src/encoder.cpp of benlaflen/bacterial-classification, unmodified, compiled
# where they lie) for one compile-time configuration, into oracle/_ref/.
# Test infrastructure only (golden vectors); needs the reference checkout.
#   sh oracle/build_ref_propagate.sh <HV_DIM> <KMER_SIZE> <SEQUENCE_LENGTH> <SIM_STEP>
set -e
# the reference checkout: $REF_ROOT, else a directory "reference" beside this repository
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF_ROOT:-$(cd "$HERE/../.." && pwd)/reference}
D=$1; K=$2; L=$3; S=$4
[ -n "$S" ] || { echo "usage: $0 DIM KMER WINDOW STEP" >&2; exit 1; }
mkdir -p "$HERE/_ref"
OUT="$HERE/_ref/propagate_D${D}_k${K}_L${L}_s${S}"
if [ -x "$OUT" ]; then echo "$OUT"; exit 0; fi
g++ -std=c++20 -O3 -march=native -ffast-math -DNORM_COSINE \
    -DREF_HV_DIM=$D -DREF_KMER=$K -DREF_WINDOW=$L -DREF_STEP=$S \
    -include "$REF/src/config.h" -include "$HERE/ref_config.h" -I"$REF/src" \
    "$REF/targets/propogate-children.cpp" "$REF/src/hierarchy.cpp" "$REF/src/HV.cpp" "$REF/src/encoder.cpp" \
    -o "$OUT.tmp"
mv "$OUT.tmp" "$OUT"
echo "$OUT"
