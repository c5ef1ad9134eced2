// Ahead-of-time kernels of the built-in Euler + Cattaneo heat-flux system
// (2 and 3 dimensions, orders 1-3).
#include "kernel_set.cuh"

namespace pypde {
namespace {
struct Reg {
  Reg() {
    register_builtin(describe<Cattaneo<2>, 1, 2, 3>("cattaneo"));
    register_builtin(describe<Cattaneo<3>, 1, 2, 3>("cattaneo"));
  }
} reg;
} // namespace
} // namespace pypde
