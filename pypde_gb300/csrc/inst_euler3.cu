// Ahead-of-time kernels of a built-in system at the order PYPDE_ORDER
// (the build compiles this unit once per order, 1-3): the Euler equations, 3-D.
#include "kernel_set.cuh"

namespace pypde {
namespace {
struct Reg {
  Reg() { register_builtin(describe<Euler<3>, PYPDE_ORDER>("euler")); }
} reg;
} // namespace
} // namespace pypde
