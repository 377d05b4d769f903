#!/bin/sh
# Build the reference's CPU path (src/HV.cpp + src/encoder.cpp of
# benlaflen/bacterial-classification, unmodified, compiled where they lie)
# together with oracle/ref_driver.cpp into oracle/_ref/, for one compile-time
# configuration.  Test infrastructure only; needs the reference checkout.
#
#   sh oracle/build_ref.sh <HV_DIM> <KMER_SIZE> <SEQUENCE_LENGTH> <SIM_STEP>
#
# Flags follow the reference's Release build (src/CMakeLists.txt:28 and
# install.sh:3): -O3 -march=native -ffast-math, NORM_COSINE on.
set -e
# the reference checkout: $REF_ROOT, else a directory "reference" beside this repository
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF_ROOT:-$(cd "$HERE/../.." && pwd)/reference}
D=$1; K=$2; L=$3; S=$4
[ -n "$S" ] || { echo "usage: $0 DIM KMER WINDOW STEP" >&2; exit 1; }
[ -f "$REF/src/HV.cpp" ] || { echo "reference sources not found under $REF" >&2; exit 3; }
mkdir -p "$HERE/_ref"
OUT="$HERE/_ref/ref_driver_D${D}_k${K}_L${L}_s${S}"
if [ -x "$OUT" ] && [ "$OUT" -nt "$HERE/ref_driver.cpp" ]; then echo "$OUT"; exit 0; fi
g++ -std=c++20 -O3 -march=native -ffast-math -DNORM_COSINE \
    -DREF_HV_DIM=$D -DREF_KMER=$K -DREF_WINDOW=$L -DREF_STEP=$S \
    -include "$REF/src/config.h" -include "$HERE/ref_config.h" \
    -I"$REF/src" \
    "$REF/src/HV.cpp" "$REF/src/encoder.cpp" "$HERE/ref_driver.cpp" \
    -o "$OUT.tmp"
mv "$OUT.tmp" "$OUT"
echo "$OUT"
