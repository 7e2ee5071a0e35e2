#!/bin/sh
# Builds oracle/_ref/ref_dump: the reference library's own basis enumeration,
# Hubbard model and compute_matrix_elements (src/algebra/*, src/utils/*),
# compiled from a copy of its sources with exactly one change:
#   src/algebra/fermion/term.h:11  term_size 32 -> 128
# The stock value caps a monomial at 7 operators, which silently drops
# every Hubbard term acting on a sector with more than 3 particles
# (src/algebra/expression_base.h:182-186); 128 gives a 55-operator cap.
# Also builds oracle/_ref/cereal_pin (oracle/cereal_pin.cpp against the
# reference's vendored cereal headers) and oracle/_ref/ref_numerics_pin
# (oracle/ref_numerics_pin.cpp: the reference's numerics/lanczos.h,
# numerics/evolve_state.h and numerics/kpm.h, unchanged and in place, with the
# Armadillo stand-in oracle/arma_shim).
# The copy and the binaries live only under oracle/_ref/ (git-ignored).
# Test infrastructure: the product never calls anything built here.
set -e
REF=${MANYBODY_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/src/algebra" ]; then
  # machines without the reference sources use the committed
  # golden fixtures instead; nothing to build
  echo "build_ref.sh: no reference sources under $REF (set MANYBODY_REFERENCE); skipped"
  exit 0
fi
rm -rf "$OUT/src"
mkdir -p "$OUT/src"
cp -r "$REF/src/algebra" "$REF/src/utils" "$OUT/src/"
sed -i 's/^constexpr size_t term_size = 32;$/constexpr size_t term_size = 128;/' \
  "$OUT/src/algebra/fermion/term.h"
grep -q '^constexpr size_t term_size = 128;$' "$OUT/src/algebra/fermion/term.h" || {
  echo "build_ref.sh: term_size patch did not apply" >&2
  exit 3
}
${CXX:-g++} -std=c++20 -O2 -fopenmp -DNDEBUG \
  -I"$OUT/src" -I"$REF/third-party" \
  "$HERE/ref_dump.cpp" \
  "$OUT/src/algebra/basis.cpp" \
  "$OUT/src/algebra/fermion/expression.cpp" \
  "$OUT/src/utils/xxhash_impl.cpp" \
  -o "$OUT/ref_dump"
echo "built $OUT/ref_dump"
# The cache-format pin: the vendored cereal library only (no reference code).
${CXX:-g++} -std=c++17 -O2 -I"$REF/third-party" "$HERE/cereal_pin.cpp" -o "$OUT/cereal_pin"
echo "built $OUT/cereal_pin"
# The numerics pin: the reference's own Lanczos, evolution and KPM code on the
# CPU, with the Armadillo stand-in (the headers are used in place, unpatched).
${CXX:-g++} -std=c++20 -O2 -I"$HERE/arma_shim" -I"$REF/src" \
  "$HERE/ref_numerics_pin.cpp" -o "$OUT/ref_numerics_pin"
echo "built $OUT/ref_numerics_pin"
