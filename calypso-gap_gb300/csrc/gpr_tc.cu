// gpr_tc.cu - tensor-core GPR (placeholder until the tcgen05 kernel lands;
// GAPGB_PREC_TC is rejected by gapgb_set_option, so this is never reached).
#include "gapgb_internal.h"

namespace gapgb {
void launch_gpr_tc(gapgb_model *m, Workspace &ws, int N, cudaStream_t st) {
  (void)m; (void)ws; (void)N; (void)st;
}
}  // namespace gapgb
