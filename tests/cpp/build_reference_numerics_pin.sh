#!/bin/sh
# Builds tests/cpp/reference_numerics_pin.cpp into $1: the reference's own
# numerics/lanczos.h and numerics/evolve_state.h, unchanged, from the
# reference's source tree, with the Armadillo stand-in in tests/cpp/arma_shim.
# The tree is MANYBODY_REFERENCE (default /root/reference); exits 77 when its
# sources are absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${MANYBODY_REFERENCE:-/root/reference}
if [ ! -f "$REF/src/numerics/lanczos.h" ]; then
  echo "no reference sources under $REF (set MANYBODY_REFERENCE)"
  exit 77
fi
exec g++ -std=c++20 -O2 -Wall -I "$HERE/arma_shim" -I "$REF/src" \
  "$HERE/reference_numerics_pin.cpp" -o "$1"
