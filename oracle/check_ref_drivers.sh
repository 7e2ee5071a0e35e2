#!/bin/sh
# Compiles tests/cpp/reference_driver_check.cpp: the reference's own
# numerics/lanczos.h and numerics/evolve_state.h (with linear_operator.h),
# unchanged, from the reference's source tree, instantiated with this
# library's mbgpu::GpuHubbardOperator<arma::cx_vec>, against the Armadillo
# stand-in in oracle/arma_shim (syntax and instantiation only: nothing is
# linked or run).  The tree is MANYBODY_REFERENCE (default /root/reference);
# exits 77 when its sources are absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/.." && pwd)
REF=${MANYBODY_REFERENCE:-/root/reference}
if [ ! -f "$REF/src/numerics/lanczos.h" ]; then
  echo "no reference sources under $REF (set MANYBODY_REFERENCE)"
  exit 77
fi
exec g++ -std=c++20 -fsyntax-only -Wall -I "$HERE/arma_shim" -I "$ROOT/include" -I "$REF/src" \
  "$ROOT/tests/cpp/reference_driver_check.cpp"
