// km_tc.cu -- tcgen05 BF16 k-means distances (placeholder).
#include "km_kernels.cuh"

namespace fem {
bool km_tc_supported(int d, int k) { return false; }
int km_tc_create(fem_km *h) { return FEM_ERR_UNSUPPORTED; }
void km_tc_destroy(fem_km *h) {}
int km_tc_upload(fem_km *h) { return FEM_ERR_UNSUPPORTED; }
int km_tc_assign(fem_km *h) { return FEM_ERR_UNSUPPORTED; }
}  // namespace fem
