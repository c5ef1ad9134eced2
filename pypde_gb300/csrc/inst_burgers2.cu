// Ahead-of-time kernels of a built-in system at the order PYPDE_ORDER
// (the build compiles this unit once per order, 1-3): the viscous Burgers
// test system (second-order form), 1-D.
#include "kernel_set.cuh"

namespace pypde {
namespace {
struct Reg {
  Reg() { register_builtin(describe<Burgers2, PYPDE_ORDER>("burgers2")); }
} reg;
} // namespace
} // namespace pypde
