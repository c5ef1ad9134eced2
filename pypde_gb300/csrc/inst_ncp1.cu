// Ahead-of-time kernels of a built-in system at the order PYPDE_ORDER
// (the build compiles this unit once per order, 1-3): the
// non-conservative test system, 1-D.
#include "kernel_set.cuh"

namespace pypde {
namespace {
struct Reg {
  Reg() { register_builtin(describe<Ncp<1>, PYPDE_ORDER>("ncp")); }
} reg;
} // namespace
} // namespace pypde
