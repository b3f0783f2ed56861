#!/usr/bin/env bash
# Builds the reference's own CPU MPM step (brocbyte/realtime-deformations) as a
# headless shared library, oracle/_ref/librd_ref.so, for use as the parity
# oracle and the timed CPU baseline.  Test infrastructure only.
#
#   usage: oracle/ref/build_ref.sh REFERENCE_ROOT   (the directory holding realtime-deformations/)
#
# Four first-party files are staged into oracle/_ref/src (git-ignored, deleted
# again once the library is linked) because three of them are patched; everything else (glm, Eigen, mcloptlib, the polar
# decomposition headers, utils.h, logger.hpp, constants.hpp) is compiled where it
# lies in the reference tree.  Each patch replaces one exact reference line and
# the script fails if a pattern does not match exactly once.
#   P1  material_point_method.hpp:155  drop the dense cells x N weight table
#       (8.6 GB at 64^3 x 8192; the live step never reads it)
#   P2  material_point_method.hpp:143,170,201  private -> public (read grid / state)
#   P3  material_point_method.cpp:237,238,240,242,260,320  material constants,
#       gravity and the clamp bounds read settable globals (defaults identical)
#   P4  material_point_method.cpp:311,323,324  glm<->Eigen conversion around the
#       plastic SVD goes through rd_ref_toEigen/rd_ref_toGlm, which reproduce
#       the reference's transposition unless rd_ref_p4 = 1
set -euo pipefail
REF_ROOT="${1:?usage: build_ref.sh REFERENCE_ROOT}"
RD="$REF_ROOT/realtime-deformations"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/../_ref"
SRC="$OUT/src"
CXX="${CXX:-g++}"

if [ ! -f "$RD/material_point_method.cpp" ]; then
    echo "build_ref.sh: reference sources not found under $RD" >&2
    exit 2
fi
mkdir -p "$SRC"
for f in material_point_method.hpp material_point_method.cpp mathy.hpp mathy.cpp; do
    cp "$RD/$f" "$SRC/$f"
    chmod u+w "$SRC/$f"
done

patch_once() {  # file, exact pattern (fixed string), replacement (sed-escaped)
    local file="$1" pat="$2" rep="$3"
    local n
    n=$(grep -cF -- "$pat" "$file" || true)
    if [ "$n" != "1" ]; then
        echo "build_ref.sh: pattern matched $n times in $(basename "$file"): $pat" >&2
        exit 3
    fi
    local esc
    esc=$(printf '%s' "$pat" | sed -e 's/[]\/$*.^[]/\\&/g')
    sed -i -e "s/$esc/$rep/" "$file"
}

H="$SRC/material_point_method.hpp"
C="$SRC/material_point_method.cpp"
# P1
patch_once "$H" 'w.resize((long long)MAX_I * MAX_J * MAX_K * nParticles);' '(void)wSize; \/* P1 *\/'
# P2 (Grid :143, WeightStorage :170 and LagrangeEulerView :201)
n=$(grep -cE '^    private:\r?$' "$H" || true)
[ "$n" = "3" ] || { echo "build_ref.sh: P2 pattern matched $n times" >&2; exit 3; }
sed -i -E -e 's/^    private:(\r?)$/    public: \/\* P2 \*\/\1/' "$H"
# P3
patch_once "$C" 'const auto poisson = 0.2f;' 'const auto poisson = rd_ref_nu;'
patch_once "$C" 'const auto E = 1.4e5f;' 'const auto E = rd_ref_E;'
patch_once "$C" 'const auto mu = mu0 * glm::exp(xi * (1 - glm::determinant(p.FPlastic)));' \
    'const auto mu = mu0 * glm::exp(rd_ref_xi * (1 - glm::determinant(p.FPlastic)));'
patch_once "$C" 'const auto lambda = lambda0 * glm::exp(xi * (1 - glm::determinant(p.FPlastic)));' \
    'const auto lambda = lambda0 * glm::exp(rd_ref_xi * (1 - glm::determinant(p.FPlastic)));'
patch_once "$C" 'glm::vec3(0, -9.8, 0)' 'glm::vec3(0, rd_ref_gy, 0)'
patch_once "$C" '(float)(1 - 2.5f * 1e-2), (float)(1 + 5.0f * 1e-3)' \
    '(float)(1 - rd_ref_theta_c), (float)(1 + rd_ref_theta_s)'
# P4
patch_once "$C" 'const auto m = glmToEigen(FEpKryshka);' 'const auto m = rd_ref_toEigen(FEpKryshka);'
patch_once "$C" 'const auto U = eigenToGlm(svd.matrixU());' 'const auto U = rd_ref_toGlm(svd.matrixU());'
patch_once "$C" 'const auto V = eigenToGlm(svd.matrixV());' 'const auto V = rd_ref_toGlm(svd.matrixV());'
patch_once "$C" '#include "cudaCalc.cuh"' '#include "cudaCalc.cuh"\n#include "rd_ref_patch.hpp"'

grep -q 'P2 \*/' "$H" || { echo "build_ref.sh: P2 not applied" >&2; exit 3; }

INC=(-I"$SRC" -I"$HERE/shim" -I"$RD" -I"$RD/include" -I"$RD/external" -I"$RD/external/glm-0.9.7.1")
FLAGS=(-std=c++17 -O2 -fPIC -ffp-contract=off -w -include "$HERE/shim/rd_ref_prelude.hpp")
rm -f "$OUT"/*.o "$OUT/librd_ref.so"
"$CXX" "${FLAGS[@]}" "${INC[@]}" -c "$C" -o "$OUT/material_point_method.o" & p1=$!
"$CXX" "${FLAGS[@]}" "${INC[@]}" -c "$SRC/mathy.cpp" -o "$OUT/mathy.o" & p2=$!
"$CXX" "${FLAGS[@]}" "${INC[@]}" -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o" & p3=$!
wait $p1; wait $p2; wait $p3
"$CXX" -shared -o "$OUT/librd_ref.so" "$OUT/material_point_method.o" "$OUT/mathy.o" "$OUT/ref_harness.o"
# keep only the library: the staged reference sources and objects are removed
rm -rf "$SRC" "$OUT"/*.o
echo "built $OUT/librd_ref.so"
