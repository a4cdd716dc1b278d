#!/bin/sh
# Test infrastructure only.  Compiles the reference's own CPU sources for the
# cross-correlation path, in place and unmodified, together with
# oracle/ref_harness.cc into oracle/_ref/libsatsuma_ref.so, and the unmodified
# reference slave (analysis/HomologyByXCorrSlave.cc) into
# oracle/_ref/HomologyByXCorrSlave.  Nothing is written outside oracle/_ref/.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
# Exits 0 without doing anything when the reference tree is absent.
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/analysis/CrossCorr.cc" ]; then
  echo "build_ref: no reference tree at $REF, skipping"
  exit 0
fi
mkdir -p "$OUT"
# The reference forgets <cstdint>/<memory> in two headers (SequenceMatch.h,
# SatsumaSynteny2.cc); force-including them is the only deviation from its
# own build flags (-O3 -std=c++14 -w).
CXXFLAGS="-O3 -std=c++14 -w -fPIC -include cstdint -include memory -I$REF"
LIBSRC="$REF/analysis/CrossCorr.cc $REF/analysis/DNAVector.cc $REF/analysis/CodonTranslate.cc \
 $REF/analysis/AlignProbability.cc $REF/analysis/ProbTable.cc $REF/base/FileParser.cc \
 $REF/base/StringUtil.cc $REF/util/mutil.cc"
g++ $CXXFLAGS -shared -o "$OUT/libsatsuma_ref.so" "$HERE/ref_harness.cc" $LIBSRC -lpthread
# The unmodified slave, for end-to-end pinning through its TCP protocol.
g++ $CXXFLAGS -o "$OUT/HomologyByXCorrSlave" "$REF/analysis/HomologyByXCorrSlave.cc" \
  "$REF/analysis/SeqChunk.cc" "$REF/analysis/SequenceMatch.cc" $LIBSRC -lpthread
echo "build_ref: wrote $OUT/libsatsuma_ref.so and $OUT/HomologyByXCorrSlave"
