// tube_cache.cuh -- factored tubes shared across calls (tube_cache.cu).
#pragma once
#include <memory>

struct sqbem_tube;

namespace sqbem {
// The tube Tube(R, L, a, n_theta, n_r, mu) in the given precision mode,
// assembled and factored on first use and then shared.  The returned tube is
// complete (its stream synchronized) and read-only; a caller that launched work
// reading it must synchronize that work before dropping its reference.
std::shared_ptr<const sqbem_tube> cached_tube(double R, double L, double a, int n_theta, int n_r, double mu,
                                              int precision);
}  // namespace sqbem
