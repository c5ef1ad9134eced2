// jit.cpp -- run-time compilation of user callback systems.
#include "../../include/pypde_gb300.h"
#include "runtime.h"

namespace pypde {

int compile_system(const char *src, const char *name, int ndim, int V,
                   int has_F, int has_B, int has_S, int second_order,
                   SystemDesc **out) {
  (void)src; (void)name; (void)ndim; (void)V; (void)has_F; (void)has_B;
  (void)has_S; (void)second_order; (void)out;
  set_error("run-time compiled callbacks are not built yet");
  return PYPDE_ERR_UNSUPPORTED;
}

void release_system(SystemDesc *d) { delete d; }

} // namespace pypde
