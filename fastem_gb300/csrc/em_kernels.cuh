// em_kernels.cuh -- launchers shared between the EM translation units.
#pragma once

#include "fem_internal.cuh"

namespace fem {

// em_plain.cu
int em_plain_estep(fem_em *h);
int em_plain_mstep(fem_em *h);
int em_factor(fem_em *h, bool regularize);
int64_t em_plain_logl_blocks(int64_t n, int d);
void cov_geometry(int d, int *TB, int *nb, int *nblk);
int em_post_rows(fem_em *h, int64_t r0, int64_t rows, double *dout);
int em_classes(fem_em *h, int32_t *dcls);

// em_tc.cu (tcgen05 mixed precision)
bool em_tc_supported(int d, int k);
int em_tc_create(fem_em *h);
void em_tc_destroy(fem_em *h);
int em_tc_upload(fem_em *h);    // X -> bf16 hi/lo split
int em_tc_prepare(fem_em *h);   // factors -> permuted bf16 hi/lo operands + offsets
int em_tc_estep(fem_em *h);
int em_tc_mstep(fem_em *h);
// the mixed path's covariance on CUDA cores in FP32 (for small components):
// posteriors as FP16 hi + lo, means as float with row stride mu_ld
int em_cov_hilo(fem_em *h, const __half *Rh, const __half *Rl, int64_t pitch, const float *muf, int mu_ld);
// true when the mixed path computes covariances with em_cov_hilo
bool em_tc_small_components(int64_t n, int k, int d);
// device posteriors of the mixed path: FP16 hi / lo, component-major, row pitch
void em_tc_posteriors(fem_em *h, const __half **rh, const __half **rl, int64_t *pitch);
// records event `slot` on the handle's stream when timing is enabled
void timing_begin(fem_em *h, int slot);
int em_tc_post_rows(fem_em *h, int64_t r0, int64_t rows, double *dout);
int em_tc_classes(fem_em *h, int32_t *dcls);
// clears the mixed kernels' bounded-wait status word
int em_tc_reset_err(fem_em *h);
// runs the bounded-wait expiry self-test kernel; *roles = bit mask of the
// waits that gave up (1 consumer, 2 drain, 4 and 8 the two flag-driven waiters)
int em_tc_wait_selftest(fem_em *h, long long budget, int *roles);

// em_wide.cu (tcgen05 split precision, 64 < d <= 256; em_tc_* dispatch here
// when the handle's d is above 64)
bool em_wide_supported(int d, int k);
int em_wide_create(fem_em *h);
void em_wide_destroy(fem_em *h);
int em_wide_upload(fem_em *h);
int em_wide_prepare(fem_em *h);
int em_wide_estep(fem_em *h);
int em_wide_mstep(fem_em *h);
int em_wide_reset_err(fem_em *h);
int em_wide_post_rows(fem_em *h, int64_t r0, int64_t rows, double *dout);
void em_wide_posteriors(fem_em *h, const __half **rh, const __half **rl, int64_t *pitch);
int em_wide_classes(fem_em *h, int32_t *dcls);

// host_linalg.cpp
// largest condition number of the K covariances (FP64 Jacobi on the device)
int em_max_cond(fem_em *h, double *cond);

}  // namespace fem
