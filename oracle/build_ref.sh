#!/bin/sh
# Test infrastructure only.  Compiles the reference's own CPU sources for the
# cross-correlation path, unmodified, together with oracle/ref_harness.cc into
# oracle/_ref/libsatsuma_ref.so, and the unmodified reference slave
# (analysis/HomologyByXCorrSlave.cc) into oracle/_ref/HomologyByXCorrSlave.
# Objects go to oracle/_ref/obj; nothing is written outside oracle/_ref/.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $SATSUMA2_REFERENCE, else the copy that
#   install_ref.sh placed in baseline/_ref/satsuma2.
# Exits 0 without doing anything when no reference tree is found.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${SATSUMA2_REFERENCE:-$HERE/../baseline/_ref/satsuma2}}
OUT="$HERE/_ref"
if [ ! -f "$REF/analysis/CrossCorr.cc" ]; then
  echo "build_ref: no reference tree at $REF, skipping"
  exit 0
fi
REF=$(cd "$REF" && pwd)
mkdir -p "$OUT/obj"
# The reference forgets <cstdint>/<memory> in two headers (SequenceMatch.h,
# SatsumaSynteny2.cc); force-including them is the only deviation from its
# own build flags (-O3 -std=c++14 -w).
CXXFLAGS="-O3 -std=c++14 -w -fPIC -include cstdint -include memory -I$REF"
LIBSRC="analysis/CrossCorr.cc analysis/DNAVector.cc analysis/CodonTranslate.cc \
 analysis/AlignProbability.cc analysis/ProbTable.cc base/FileParser.cc base/StringUtil.cc util/mutil.cc"
SLAVESRC="analysis/HomologyByXCorrSlave.cc analysis/SeqChunk.cc analysis/SequenceMatch.cc"
# one compiler process per translation unit, all at once
pids=""
for s in $LIBSRC $SLAVESRC; do
  o="$OUT/obj/$(echo "$s" | tr '/' '_').o"
  g++ $CXXFLAGS -c "$REF/$s" -o "$o" &
  pids="$pids $!"
done
g++ $CXXFLAGS -c "$HERE/ref_harness.cc" -o "$OUT/obj/ref_harness.o" &
pids="$pids $!"
fail=0
for p in $pids; do
  wait "$p" || fail=1
done
[ "$fail" = 0 ] || { echo "build_ref: compile failed"; exit 1; }
LIBOBJ=""
for s in $LIBSRC; do LIBOBJ="$LIBOBJ $OUT/obj/$(echo "$s" | tr '/' '_').o"; done
SLAVEOBJ=""
for s in $SLAVESRC; do SLAVEOBJ="$SLAVEOBJ $OUT/obj/$(echo "$s" | tr '/' '_').o"; done
g++ -shared -o "$OUT/libsatsuma_ref.so.tmp" "$OUT/obj/ref_harness.o" $LIBOBJ -lpthread
mv "$OUT/libsatsuma_ref.so.tmp" "$OUT/libsatsuma_ref.so"
# The unmodified slave, for end-to-end pinning through its TCP protocol.
g++ -o "$OUT/HomologyByXCorrSlave.tmp" $SLAVEOBJ $LIBOBJ -lpthread
mv "$OUT/HomologyByXCorrSlave.tmp" "$OUT/HomologyByXCorrSlave"
echo "build_ref: wrote $OUT/libsatsuma_ref.so and $OUT/HomologyByXCorrSlave from $REF"
