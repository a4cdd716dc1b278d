#!/bin/sh
# Test infrastructure only.  Installs the reference's CPU sources for the
# cross-correlation path, unmodified, into baseline/_ref/satsuma2 (git-ignored):
# the directories analysis/, base/, util/ and extern/ of the satsuma2 tree.
# build_ref.sh compiles them from there, so the compiled reference can be
# rebuilt on a machine that has the repository but not the reference tree
# (the reference is C++ with no Python packaging, so there is no pip install).
#
# Usage: oracle/install_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $SATSUMA2_REFERENCE, else /root/reference.
# Exits 0 without doing anything when that tree is absent.
set -e
REF=${1:-${SATSUMA2_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
DEST="$HERE/../baseline/_ref/satsuma2"
if [ ! -f "$REF/analysis/CrossCorr.cc" ]; then
  echo "install_ref: no reference tree at $REF, skipping"
  exit 0
fi
mkdir -p "$DEST"
for d in analysis base util extern; do
  rm -rf "$DEST/$d"
  cp -R "$REF/$d" "$DEST/$d"
done
chmod -R u+w "$DEST"
echo "install_ref: copied analysis/ base/ util/ extern/ from $REF to $DEST"
