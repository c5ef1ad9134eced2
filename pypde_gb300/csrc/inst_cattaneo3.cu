// Ahead-of-time kernels of a built-in system at the order PYPDE_ORDER
// (the build compiles this unit once per order, 1-3): the
// Euler + Cattaneo heat-flux system, 3-D.
#include "kernel_set.cuh"

namespace pypde {
namespace {
struct Reg {
  Reg() { register_builtin(describe<Cattaneo<3>, PYPDE_ORDER>("cattaneo")); }
} reg;
} // namespace
} // namespace pypde
