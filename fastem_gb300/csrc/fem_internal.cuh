// fem_internal.cuh -- shared definitions of the sm_103a EM / k-means library.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <random>

#include "../../include/fastem_gpu.h"

namespace fem {

// thread-local message of the last failing call (fem_last_error)
void set_error(const char *fmt, ...);

// Lets `func` launch with `bytes` of dynamic shared memory on the current
// device.  The limit is a per-kernel attribute shared by every host thread, so
// it is only ever raised (under a lock): a concurrent handle that needs less
// never lowers it beneath another's launch of the same kernel.
cudaError_t allow_dyn_smem(const void *func, size_t bytes);
template <class F>
cudaError_t allow_dyn_smem(F *func, size_t bytes) {
  return allow_dyn_smem((const void *)func, bytes);
}

#define FEM_CUDA(call)                                                                  \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      ::fem::set_error("%s:%d %s failed: %s", __FILE__, __LINE__, #call,                \
                       cudaGetErrorString(e_));                                         \
      return FEM_ERR_CUDA;                                                              \
    }                                                                                   \
  } while (0)

#define FEM_TRY(expr)                 \
  do {                                \
    int s_ = (expr);                  \
    if (s_ != FEM_OK) return s_;      \
  } while (0)

// Checks that `device` exists and is an sm_103 part; selects it.
int select_device(int device);

// 2-D row-major tensor map (cols contiguous, rows pitch_bytes apart; 0 =
// packed), resolved without linking libcuda
int encode_tmap_2d(CUtensorMap *m, CUtensorMapDataType dt, int elem_bytes, const void *base, uint64_t cols,
                   uint64_t rows, uint32_t box_cols, uint32_t box_rows, CUtensorMapSwizzle swz,
                   uint64_t pitch_bytes = 0);

constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs (grids are sized from the live count)
int sm_count();

template <typename T>
int dalloc(T **p, size_t count) {
  *p = nullptr;
  if (count == 0) return FEM_OK;
  cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
  if (e != cudaSuccess) {
    set_error("cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
    *p = nullptr;
    return FEM_ERR_CUDA;
  }
  return FEM_OK;
}

template <typename T>
void dfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

// ---------------------------------------------------------------- device status
// One word per handle on the device.  Kernels never trap: they record what
// went wrong here and return; the host reads it after the sweep.
struct DevStatus {
  double logl;         // sum_i LSE_i of the last E-step
  int chol_failed;     // first component whose Cholesky pivot was <= 0 (INT_MAX: none)
  int timeout;         // a bounded wait gave up (mixed-precision kernels)
  int64_t rechecked;   // k-means rows re-decided in FP64
  double fit;          // k-means sum of squared distances
  int track_changes;   // k-means: compare each new label with the stored one (set by the host)
  int changed;         // k-means: some label differs from the stored one
  double cond_bound;   // EM: max over components of ||Sigma_j||_F ||L_j^-1||_F^2 (>= cond(Sigma_j))
};

// ------------------------------------------------------------------ EM handle
enum { EM_PAR_CHUNKS = 0 };

struct EmHandle;
struct TcEmPlan;    // mixed-precision launch plan, d <= 64 (em_tc.cu)
struct WideEmPlan;  // mixed-precision launch plan, 64 < d <= 256 (em_wide.cu)

}  // namespace fem

struct fem_em {
  int d = 0, k = 0;
  int64_t n = 0;
  fem_em_config cfg{};
  cudaStream_t stream = nullptr;
  bool have_data = false, have_params = false, have_post = false, factored = false;

  // dataset
  float *X = nullptr;                // n x d
  __half *Xhi = nullptr;             // n x d  fp16(x)        (mixed)
  __half *Xlo = nullptr;             // n x d  fp16(x - xhi)  (mixed)

  // parameters (FP64)
  double *pi = nullptr, *mu = nullptr, *sigma = nullptr;   // k, k*d, k*d*d
  double *linv = nullptr;            // k*d*d  L^-1 (lower), row-major
  double *logdet = nullptr, *logc = nullptr;  // k
  double *work = nullptr;            // k*d*d  factorisation scratch

  // kernel-side copies: T = double (FP64) or float (FP32 / mixed)
  void *muT = nullptr, *linvT = nullptr, *logcT = nullptr;

  // posteriors, component-major k x n (T)
  void *R = nullptr;

  // E-step partials
  double *logl_part = nullptr;
  int64_t n_logl_part = 0;
  // M-step partials (FP64)
  double *mpart = nullptr;      // means: grid x k x (d+1)
  int mgrid = 0;
  double *cpart = nullptr;      // covariances: chunks x k x nblk x 64
  int cchunks = 0, cunits_blocks = 0;
  double *psum = nullptr;       // k   PosteriorSum

  // mixed-precision state (em_tc.cu)
  fem::TcEmPlan *tc = nullptr;
  fem::WideEmPlan *wide = nullptr;

  fem::DevStatus *dstat = nullptr;   // device
  fem::DevStatus *hstat = nullptr;   // pinned host

  // timing
  bool timing = false;
  unsigned tmask = 0;            // event slots recorded since the last sync
  cudaEvent_t ev[10] = {};       // 0/1 E-step, 2/3 M-step, 4/5 factorisation, 6/7 train, 8/9 covariance kernel
  double t_estep = 0, t_mstep = 0, t_final = 0, t_train = 0, t_cov = 0;
  int64_t launches = 0, sweeps = 0;
};

struct fem_km {
  int d = 0, k = 0;
  int64_t n = 0;
  fem_km_config cfg{};
  cudaStream_t stream = nullptr;
  bool have_data = false;
  std::mt19937_64 rng;
  std::uniform_real_distribution<> uni;
  int64_t next_repair = 0;         // next row of FEM_KM_REPAIR_NEXT

  float *X = nullptr;              // n x d
  __nv_bfloat16 *Xb = nullptr;     // n x d (mixed)
  float *xnorm = nullptr;          // n   ||x_i|| (mixed bound)
  int32_t *labels = nullptr;       // n
  double *cent = nullptr;          // k x d (FP64 centroids, device)
  float *centf = nullptr;          // k x d float copy
  __nv_bfloat16 *centb = nullptr;  // k x d bf16 copy (mixed)
  float *cnorm = nullptr;          // k   ||c_j|| and ||c_j||^2
  long long *acc = nullptr;        // grid x k x d  fixed-point partial sums
  int *cnt = nullptr;              // grid x k
  int grid = 0;
  int shift = 0;                   // fixed-point scale 2^shift
  double xg2 = 0.0;                // sum_i ||x_i - g||^2
  double *g = nullptr;             // data mean (device, d)
  double *hg = nullptr;            // data mean (host)
  double *out = nullptr;           // device: k x d new centroids, k counts (as double), fit
  double *hout = nullptr;          // pinned host copy
  fem::DevStatus *dstat = nullptr;
  fem::DevStatus *hstat = nullptr;
  cudaEvent_t ev[4] = {};
  double t_assign = 0, t_update = 0;
  void *tc = nullptr;              // tensor-core plan (km_tc.cu)
};
