// Ahead-of-time kernels of the small test systems: the non-conservative
// Ncp system (1 and 2 dimensions) and second-order viscous Burgers (1-D).
#include "kernel_set.cuh"

namespace pypde {
namespace {
struct Reg {
  Reg() {
    register_builtin(describe<Ncp<1>, 1, 2, 3>("ncp"));
    register_builtin(describe<Ncp<2>, 1, 2, 3>("ncp"));
    register_builtin(describe<Burgers2, 1, 2, 3>("burgers2"));
  }
} reg;
} // namespace
} // namespace pypde
