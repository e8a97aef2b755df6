// em_corr.cu -- EMAlgorithm::ComputePosterriorCorrelation
// (EM2/EMAlgorithm.cpp:213-219): Corr = R^T R, K x K, over the posteriors of
// the last E-step, which stay resident on the device (component-major).
//
// 64 x 64 tiles of Corr x chunks of points; a thread owns 4 x 4 entries.
// Products of 32-point sub-blocks are summed in the accumulation type of the
// handle's precision (FP32 for FP32 / mixed, FP64 for FP64) and added to FP64
// per-thread sums; the chunks' FP64 partials are reduced in a fixed order.
#include <algorithm>

#include "em_kernels.cuh"
#include "fem_internal.cuh"

namespace fem {
namespace {

constexpr int kCorrTile = 64;
constexpr int kCorrSub = 32;

// posterior (component j, point i)
struct PostPlainF {
  const float *R;
  int64_t pitch;
  __device__ float operator()(int j, int64_t i) const { return R[(size_t)j * pitch + i]; }
};
struct PostPlainD {
  const double *R;
  int64_t pitch;
  __device__ double operator()(int j, int64_t i) const { return R[(size_t)j * pitch + i]; }
};
struct PostSplit {   // mixed precision: FP16 hi + lo
  const __half *Rh, *Rl;
  int64_t pitch;
  __device__ float operator()(int j, int64_t i) const {
    const size_t o = (size_t)j * pitch + i;
    return __half2float(Rh[o]) + __half2float(Rl[o]);
  }
};

template <class T, class Src>
__global__ void __launch_bounds__(256)
k_post_corr(Src src, int64_t n, int K, int64_t chunk, double *__restrict__ part) {
  __shared__ __align__(16) T Ra[kCorrSub][kCorrTile];
  __shared__ __align__(16) T Rb[kCorrSub][kCorrTile];
  const int t = threadIdx.x, ta = t >> 4, tb = t & 15;
  const int a0 = blockIdx.x * kCorrTile, b0 = blockIdx.y * kCorrTile;
  const int64_t i0 = (int64_t)blockIdx.z * chunk, i1 = std::min<int64_t>(n, i0 + chunk);
  double acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; u++)
#pragma unroll
    for (int v = 0; v < 4; v++) acc[u][v] = 0.0;
  for (int64_t ib = i0; ib < i1; ib += kCorrSub) {
    __syncthreads();
    for (int e = t; e < kCorrTile * kCorrSub; e += 256) {
      const int row = e / kCorrSub, p = e - row * kCorrSub;
      const int64_t i = ib + p;
      Ra[p][row] = (a0 + row < K && i < i1) ? (T)src(a0 + row, i) : (T)0;
      Rb[p][row] = (b0 + row < K && i < i1) ? (T)src(b0 + row, i) : (T)0;
    }
    __syncthreads();
    T s[4][4];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
      for (int v = 0; v < 4; v++) s[u][v] = (T)0;
#pragma unroll 4
    for (int p = 0; p < kCorrSub; p++) {
      T ra[4], rb[4];
#pragma unroll
      for (int u = 0; u < 4; u++) ra[u] = Ra[p][4 * ta + u], rb[u] = Rb[p][4 * tb + u];
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) s[u][v] += ra[u] * rb[v];
    }
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
      for (int v = 0; v < 4; v++) acc[u][v] += (double)s[u][v];
  }
#pragma unroll
  for (int u = 0; u < 4; u++)
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const int a = a0 + 4 * ta + u, b = b0 + 4 * tb + v;
      if (a < K && b < K) part[((size_t)blockIdx.z * K + a) * K + b] = acc[u][v];
    }
}

__global__ void k_corr_reduce(const double *__restrict__ part, int chunks, int K, double *__restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)K * K) return;
  double s = 0.0;
  for (int c = 0; c < chunks; c++) s += part[(size_t)c * K * K + e];
  out[e] = s;
}

template <class T, class Src>
int launch_corr(fem_em *h, Src src, double *dout) {
  const int K = h->k;
  const int tiles = (K + kCorrTile - 1) / kCorrTile;
  int64_t chunks = std::max<int64_t>(1, (int64_t)4 * sm_count() / (tiles * tiles));
  chunks = std::min<int64_t>(chunks, (h->n + 4095) / 4096);
  const int64_t chunk = (h->n + chunks - 1) / chunks;
  double *part = nullptr;
  FEM_TRY(dalloc(&part, (size_t)chunks * K * K));
  k_post_corr<T, Src><<<dim3(tiles, tiles, (unsigned)chunks), 256, 0, h->stream>>>(src, h->n, K, chunk, part);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_corr_reduce<<<(unsigned)(((int64_t)K * K + 255) / 256), 256, 0, h->stream>>>(part, (int)chunks, K, dout);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  dfree(part);
  if (e != cudaSuccess) {
    set_error("posterior correlation failed: %s", cudaGetErrorString(e));
    return FEM_ERR_CUDA;
  }
  return FEM_OK;
}

}  // namespace
}  // namespace fem

using namespace fem;

extern "C" int fem_em_posterior_correlation(fem_em *h, double *corr) {
  if (!h || !corr) {
    set_error("fem_em_posterior_correlation: null argument");
    return FEM_ERR_BAD_ARG;
  }
  if (!h->have_post) {
    set_error("no posteriors (run an E-step first)");
    return FEM_ERR_STATE;
  }
  FEM_CUDA(cudaSetDevice(h->cfg.device));
  const int K = h->k;
  double *dout = nullptr;
  FEM_TRY(dalloc(&dout, (size_t)K * K));
  int st;
  if (h->cfg.precision == FEM_PREC_MIXED) {
    const __half *rh = nullptr, *rl = nullptr;
    int64_t pitch = 0;
    em_tc_posteriors(h, &rh, &rl, &pitch);
    st = launch_corr<float>(h, PostSplit{rh, rl, pitch}, dout);
  } else if (h->cfg.precision == FEM_PREC_FP64) {
    st = launch_corr<double>(h, PostPlainD{(const double *)h->R, h->n}, dout);
  } else {
    st = launch_corr<float>(h, PostPlainF{(const float *)h->R, h->n}, dout);
  }
  if (st == FEM_OK &&
      cudaMemcpy(corr, dout, (size_t)K * K * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("posterior correlation read-back failed");
    st = FEM_ERR_CUDA;
  }
  dfree(dout);
  return st;
}
