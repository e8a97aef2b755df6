// km_kernels.cuh -- launchers shared between the k-means translation units.
#pragma once

#include "fem_internal.cuh"

namespace fem {

// km.cu
int km_launch_assign_f32(fem_km *h);
size_t km_assign_smem(int K, int D);

// km_tc.cu (tcgen05 BF16 distances)
bool km_tc_supported(int d, int k);
int km_tc_create(fem_km *h);
void km_tc_destroy(fem_km *h);
int km_tc_assign(fem_km *h);

}  // namespace fem
