// Ahead-of-time kernels of the built-in Euler system (1-3 dimensions,
// orders 1-3).
#include "kernel_set.cuh"

namespace pypde {
namespace {
struct Reg {
  Reg() {
    register_builtin(describe<Euler<1>, 1, 2, 3>("euler"));
    register_builtin(describe<Euler<2>, 1, 2, 3>("euler"));
    register_builtin(describe<Euler<3>, 1, 2, 3>("euler"));
  }
} reg;
} // namespace
} // namespace pypde
