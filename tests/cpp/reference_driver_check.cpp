// Compile check: the reference's own drivers (numerics/lanczos.h,
// numerics/evolve_state.h and numerics/linear_operator.h, unchanged, from the
// reference's source tree) instantiated with this library's
// mbgpu::GpuHubbardOperator<arma::cx_vec>.  Built with -fsyntax-only against
// a minimal Armadillo stand-in (oracle/arma_shim) by
// oracle/check_ref_drivers.sh; it is not linked or run.
#include "manybody_gb300.hpp"

#include "numerics/evolve_state.h"
#include "numerics/lanczos.h"

using Op = mbgpu::GpuHubbardOperator<arma::cx_vec>;

void drivers(const Op& op, const arma::cx_vec& b) {
  // find_min_eigenpair builds Negated<Op>(op) by value: Op must be copyable
  auto lo = find_min_eigenpair(op, 200);
  auto hi = find_max_eigenpair(op, 200);
  (void)lo;
  (void)hi;
  auto decomp = lanczos_pass_one(op, b, 20);
  std::vector<double> y(decomp.steps_taken, 1.0);
  arma::cx_vec x = lanczos_pass_two(op, b, decomp, y);
  (void)x;
  auto seed = make_seed_vector(op);
  (void)seed;
  Negated<Op> neg(op);
  Scaled<Op> sc(op, Op::ScalarType(2.0));
  Shifted<Op> sh(op, Op::ScalarType(-1.0));
  (void)neg.apply(b);
  (void)sc.apply(b);
  (void)sh.apply(b);
  // time evolution (evolve_state.h:164-231)
  EvolutionOptions opts{};
  opts.krylov_steps = 30;
  auto a = time_evolve_state(op, b, 0.1, opts);
  auto c = imaginary_time_evolve_state(op, b, 0.1);
  auto d = time_evolve_state_steps(op, b, 0.0, 1.0, 0.1);
  (void)a;
  (void)c;
  (void)d;
}
