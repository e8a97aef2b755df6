// em_tc.cu -- tcgen05 mixed-precision EM sweep (placeholder until the
// tensor-core kernels land).
#include "em_kernels.cuh"

namespace fem {
bool em_tc_supported(int d, int k) { return false; }
int em_tc_create(fem_em *h) { set_error("mixed precision not built"); return FEM_ERR_UNSUPPORTED; }
void em_tc_destroy(fem_em *h) {}
int em_tc_upload(fem_em *h) { return FEM_ERR_UNSUPPORTED; }
int em_tc_prepare(fem_em *h) { return FEM_ERR_UNSUPPORTED; }
int em_tc_estep(fem_em *h) { return FEM_ERR_UNSUPPORTED; }
int em_tc_mstep(fem_em *h) { return FEM_ERR_UNSUPPORTED; }
}  // namespace fem
