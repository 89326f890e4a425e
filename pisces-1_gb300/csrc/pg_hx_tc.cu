// Mixed-precision H*X (split-TF32 tensor-core kinetic contractions): placeholder
// until the tcgen05 kernel lands.
#include "pg_common.cuh"

namespace pg {
pg_status hx_mixed(const pg_grid* g, const double* v, const double* x, double* y, int nvec, cudaStream_t st) {
  (void)g; (void)v; (void)x; (void)y; (void)nvec; (void)st;
  set_error("pg_hx: mixed precision is not built yet");
  return PG_UNSUPPORTED;
}
}  // namespace pg
