#!/usr/bin/env bash
# Copies the reference sources that build_ref.sh compiles into
# oracle/_ref/tree/realtime-deformations (git-ignored, never committed), so that
# the headless reference can be built on a machine that has no checkout of the
# reference - the Arm host that runs the GPU measurements - by
#   oracle/ref/build_ref.sh oracle/_ref/tree
# Test infrastructure only (the CPU baseline and the oracle).
#
#   usage: oracle/ref/stage_tree.sh REFERENCE_ROOT   (the directory holding realtime-deformations/)
#
# Copied: the first-party files and headers that the three translation units
# include (found with g++ -MM), and the header-only libraries they use whole -
# Eigen and glm choose architecture-specific headers when compiled, so the
# x86 dependency list alone would not build on Arm.
set -euo pipefail
REF_ROOT="${1:?usage: stage_tree.sh REFERENCE_ROOT}"
RD="$REF_ROOT/realtime-deformations"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
TREE="$HERE/../_ref/tree"
DST="$TREE/realtime-deformations"
CXX="${CXX:-g++}"

if [ ! -f "$RD/material_point_method.cpp" ]; then
    echo "stage_tree.sh: reference sources not found under $RD" >&2
    exit 2
fi
INC=(-I"$HERE/shim" -I"$RD" -I"$RD/include" -I"$RD/external" -I"$RD/external/glm-0.9.7.1")
deps=$("$CXX" -std=c++17 -MM "${INC[@]}" -include "$HERE/shim/rd_ref_prelude.hpp" \
       "$RD/material_point_method.cpp" "$RD/mathy.cpp" "$HERE/ref_harness.cpp" | tr ' \\' '\n\n' | grep -F "$RD/" | sort -u)
rm -rf "$TREE"
mkdir -p "$DST"
for f in $deps material_point_method.cpp mathy.cpp; do
    rel="${f#"$RD/"}"
    mkdir -p "$DST/$(dirname "$rel")"
    cp "$RD/$rel" "$DST/$rel"
done
mkdir -p "$DST/external/glm-0.9.7.1"
cp -r "$RD/external/Eigen" "$DST/external/"
cp -r "$RD/external/glm-0.9.7.1/glm" "$DST/external/glm-0.9.7.1/"
chmod -R u+w "$TREE"
echo "staged $(find "$DST" -type f | wc -l) files into $TREE"
