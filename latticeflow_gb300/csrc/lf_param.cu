// Parametric flow / TV driver (filled in below).
#include "lf_engine.h"

namespace lfg {
void engine_run_parametric(Engine&) { throw LfError{8, "parametric solve not built yet"}; }
int tv_2d(const KernelDef*, size_t, size_t, const double*, double, double*, int64_t*) { return 8; }
}  // namespace lfg
