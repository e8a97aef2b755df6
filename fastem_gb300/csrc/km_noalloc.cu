// km_noalloc.cu -- k-means classification that allocates nothing:
// CentroidVector::ClassifyDataset + ComputeMSE (Clust/CentroidVector.cpp:8-34,
// 56-94) on caller-owned device buffers, without a handle.
//
// Who needs it: callers that own their whole device-memory budget and must
// not allocate once they are running -- a long-lived service that labels
// incoming batches in buffers it sized up front, or a caller sharing the GPU
// with other streams, where a cudaMalloc / cudaFree could synchronise the
// device and stall the others.  The handle API (fem_km_create) allocates its
// working set at creation; this entry point instead keeps its few scratch
// values in one file-scope __device__ array of fixed size.
//
// Scratch (g_na_scratch, 140 KiB): the FP32 copy of the centroids (k*d
// floats, k*d <= 32768), their norms (k <= 1024 floats) and one FP64 fit
// partial per CTA (<= 1024).  Larger k or k*d are rejected with
// FEM_ERR_BAD_ARG and a message naming the limit.
//
// Sharing: every call on a device uses the same array.  It keeps whatever
// the last call left there; nothing in it has to start at zero, because each
// call writes every entry it later reads (centroid copy, norms, one partial
// per CTA of this call's grid) before reading it.  Two calls that overlap in
// time on the same device -- on different streams, or from different host
// threads -- race on the array and may return wrong labels or fits; callers
// must order them (one stream, or events).
//
// Set-up: the first call on a device makes that device current for a moment
// and resolves the array's device address with cudaGetSymbolAddress (which
// can load this library's device code onto the device), reads the SM count
// and raises the kernels' shared-memory limit.  That first call should
// therefore come before any stream capture the caller may start.  Later calls
// only launch three kernels on the given stream.
#include <cfloat>
#include <climits>
#include <cmath>
#include <mutex>

#include "fem_internal.cuh"

namespace fem {
namespace {

constexpr int kNaMaxKD = 32768;    // k * d
constexpr int kNaMaxK = 1024;
constexpr int kNaMaxGrid = 1024;   // CTAs (one FP64 partial each)
constexpr int kNaRows = 256;       // rows per tile (one per thread)
constexpr size_t kNaScratchBytes = (size_t)kNaMaxKD * 4 + (size_t)kNaMaxK * 4 + (size_t)kNaMaxGrid * 8;
constexpr int kNaMaxDevices = 64;

__device__ __align__(256) unsigned char g_na_scratch[kNaScratchBytes];

struct NaScratch {
  float *centf;    // k x d
  float *cnorm;    // k
  double *part;    // grid
};

__host__ __device__ inline NaScratch na_layout(void *base) {
  unsigned char *b = static_cast<unsigned char *>(base);
  return NaScratch{reinterpret_cast<float *>(b), reinterpret_cast<float *>(b + (size_t)kNaMaxKD * 4),
                   reinterpret_cast<double *>(b + (size_t)kNaMaxKD * 4 + (size_t)kNaMaxK * 4)};
}

// FP32 centroid copy and norms
__global__ void k_na_prep(const double *__restrict__ cent, int K, int d, float *__restrict__ centf,
                          float *__restrict__ cnorm) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K) return;
  double s = 0.0;
  for (int q = 0; q < d; q++) {
    const double c = cent[(size_t)j * d + q];
    centf[(size_t)j * d + q] = (float)c;
    s += c * c;
  }
  cnorm[j] = (float)sqrt(s);
}

// FP64 difference form in column order without contraction (the reference's
// per-point squared distance, bit for bit)
__device__ __forceinline__ double na_dist64(const double *__restrict__ c, const float *x, int d) {
  double s = 0.0;
  for (int q = 0; q < d; q++) {
    const double t = __dsub_rn(c[q], (double)x[q]);
    s = __dadd_rn(s, __dmul_rn(t, t));
  }
  return s;
}

// bound on |FP32 difference-form distance - exact distance|, doubled
__device__ __forceinline__ float na_bound(float s, float cn, int d) {
  const float u = 5.9604645e-8f;  // 2^-24
  return 2.f * ((float)(d + 4) * u * s + 2.01f * u * sqrtf(fmaxf(s, 0.f)) * cn + u * u * cn * cn) +
         1e-30f;
}

// One thread per row of a 256-row tile: FP32 distances to every centroid
// with an error bound; rows whose winner is not separated by the bounds are
// decided in FP64 (index order, strict <).  The winner's FP64 distance is
// added to the thread's fit sum; the CTA's sum goes to part[blockIdx.x].
template <int D>
__global__ void __launch_bounds__(kNaRows)
k_na_classify(const float *__restrict__ X, int64_t n, int K, const float *__restrict__ centf,
              const float *__restrict__ cnorm, const double *__restrict__ cent, int32_t *__restrict__ labels,
              double *__restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem_na[];
  float *sC = reinterpret_cast<float *>(smem_na);   // K x D
  float *sCn = sC + (size_t)K * D;                   // K
  float *sX = sCn + K;                               // 256 x (D + 1)
  __shared__ double red[kNaRows / 32];
  const int tid = threadIdx.x;
  for (int e = tid; e < K * D; e += kNaRows) sC[e] = centf[e];
  for (int j = tid; j < K; j += kNaRows) sCn[j] = cnorm[j];
  double fit = 0.0;
  const int64_t ntiles = (n + kNaRows - 1) / kNaRows;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t base = tile * kNaRows;
    const int rows = (int)min((int64_t)kNaRows, n - base);
    __syncthreads();
    for (int e = tid; e < rows * D; e += kNaRows) {
      const int p = e / D, q = e - p * D;
      sX[p * (D + 1) + q] = X[base * D + e];
    }
    __syncthreads();
    if (tid < rows) {
      float x[D];
#pragma unroll
      for (int q = 0; q < D; q++) x[q] = sX[tid * (D + 1) + q];
      float U = INFINITY, lb1 = INFINITY, lb2 = INFINITY;
      int j1 = 0;
      for (int j = 0; j < K; j++) {
        const float *c = sC + j * D;
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < D; q++) {
          const float t = x[q] - c[q];
          s = fmaf(t, t, s);
        }
        const float b = na_bound(s, sCn[j], D);
        U = fminf(U, s + b);
        if (s - b < lb1) {
          lb2 = lb1;
          lb1 = s - b;
          j1 = j;
        } else if (s - b < lb2) {
          lb2 = s - b;
        }
      }
      int lab = j1;
      double best;
      if (lb2 > U) {
        best = na_dist64(cent + (size_t)j1 * D, x, D);
      } else {
        // candidates within the bound, decided in FP64; a row whose FP32
        // distances are not finite (NaN, or beyond FP32 range) has no
        // candidate and is decided over every centroid, so it gets the
        // reference's answer: label -1 and DBL_MAX where no distance is
        // below DBL_MAX (a NaN row)
        lab = -1;
        best = DBL_MAX;
        for (int j = 0; j < K; j++) {
          const float *c = sC + j * D;
          float s = 0.f;
#pragma unroll
          for (int q = 0; q < D; q++) {
            const float t = x[q] - c[q];
            s = fmaf(t, t, s);
          }
          if (s - na_bound(s, sCn[j], D) <= U) {
            const double s64 = na_dist64(cent + (size_t)j * D, x, D);
            if (s64 < best) {
              best = s64;
              lab = j;
            }
          }
        }
        if (lab < 0)
          for (int j = 0; j < K; j++) {
            const double s64 = na_dist64(cent + (size_t)j * D, x, D);
            if (s64 < best) {
              best = s64;
              lab = j;
            }
          }
      }
      labels[base + tid] = lab;
      fit += best;
    }
  }
  // fixed-order CTA sum
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) fit += __shfl_down_sync(0xffffffffu, fit, o);
  if ((tid & 31) == 0) red[tid >> 5] = fit;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < kNaRows / 32; w++) s += red[w];
    part[blockIdx.x] = s;
  }
}

// fit = (sum of the CTA partials in index order) / n
__global__ void k_na_final(const double *__restrict__ part, int G, int64_t n, double *__restrict__ fit) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < G; b++) s += part[b];
    *fit = s / (double)n;
  }
}

size_t na_smem(int K, int D) { return ((size_t)K * D + K + (size_t)kNaRows * (D + 1)) * 4; }

struct NaDevice {
  void *scratch = nullptr;
  int sms = 0;
};
std::mutex g_na_mu;
NaDevice g_na_dev[kNaMaxDevices];

template <int D>
cudaError_t na_raise_smem() {
  return cudaFuncSetAttribute(k_na_classify<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)na_smem(kNaMaxKD / D < kNaMaxK ? kNaMaxKD / D : kNaMaxK, D));
}

// first call per device: scratch address, SM count, shared-memory limits
int na_setup(int device, NaDevice *out) {
  std::lock_guard<std::mutex> lock(g_na_mu);
  NaDevice &nd = g_na_dev[device];
  if (nd.scratch) {
    *out = nd;
    return FEM_OK;
  }
  int prev = 0;
  FEM_CUDA(cudaGetDevice(&prev));
  if (prev != device) FEM_CUDA(cudaSetDevice(device));
  int sms = 0, major = 0, minor = 0;
  cudaError_t e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
  if (e == cudaSuccess && (major != 10 || minor != 3)) {
    if (prev != device) cudaSetDevice(prev);
    set_error("device %d is sm_%d%d; this library is built for sm_103 (GB300) only", device, major, minor);
    return FEM_ERR_NO_DEVICE;
  }
  void *p = nullptr;
  if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_na_scratch);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = na_raise_smem<2>();
  if (e == cudaSuccess) e = na_raise_smem<4>();
  if (e == cudaSuccess) e = na_raise_smem<8>();
  if (e == cudaSuccess) e = na_raise_smem<16>();
  if (e == cudaSuccess) e = na_raise_smem<32>();
  if (e == cudaSuccess) e = na_raise_smem<64>();
  if (prev != device) cudaSetDevice(prev);
  if (e != cudaSuccess) {
    set_error("k-means classification set-up on device %d failed: %s", device, cudaGetErrorString(e));
    return FEM_ERR_CUDA;
  }
  nd.scratch = p;
  nd.sms = sms;
  *out = nd;
  return FEM_OK;
}

}  // namespace
}  // namespace fem

using namespace fem;

extern "C" int fem_km_classify_noalloc(int d, int64_t n, int k, const float *dX, const double *dCent,
                                       int32_t *dLabels, double *dFit, int device, void *stream) {
  if (!dX || !dCent || !dLabels || !dFit) {
    set_error("fem_km_classify_noalloc: null device pointer");
    return FEM_ERR_BAD_ARG;
  }
  if (n < 1 || k < 1) {
    set_error("fem_km_classify_noalloc: need n >= 1 and k >= 1 (got n=%lld, k=%d)", (long long)n, k);
    return FEM_ERR_BAD_ARG;
  }
  if (d != 2 && d != 4 && d != 8 && d != 16 && d != 32 && d != 64) {
    set_error("fem_km_classify_noalloc: d must be one of 2, 4, 8, 16, 32, 64 (got %d)", d);
    return FEM_ERR_UNSUPPORTED;
  }
  if (k > kNaMaxK || (int64_t)k * d > kNaMaxKD) {
    set_error("fem_km_classify_noalloc: k=%d, d=%d exceeds the fixed scratch (k <= %d and k*d <= %d)", k, d,
              kNaMaxK, kNaMaxKD);
    return FEM_ERR_BAD_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    set_error("fem_km_classify_noalloc: no CUDA device");
    return FEM_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev || device >= kNaMaxDevices) {
    set_error("fem_km_classify_noalloc: device %d out of range", device);
    return FEM_ERR_BAD_ARG;
  }
  // an error left pending by earlier work of the caller would otherwise be
  // read back below as this call's launch failure: report it as what it is
  // (and leave it pending for the caller)
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess) {
    set_error("fem_km_classify_noalloc: a CUDA error was already pending before this call: %s",
              cudaGetErrorString(pending));
    return FEM_ERR_CUDA;
  }
  NaDevice nd;
  FEM_TRY(na_setup(device, &nd));
  const NaScratch S = na_layout(nd.scratch);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int prev = 0;
  FEM_CUDA(cudaGetDevice(&prev));
  if (prev != device) FEM_CUDA(cudaSetDevice(device));
  const int64_t ntiles = (n + kNaRows - 1) / kNaRows;
  const int grid = (int)std::min<int64_t>(ntiles, std::min(nd.sms, kNaMaxGrid));
  k_na_prep<<<(k + 127) / 128, 128, 0, st>>>(dCent, k, d, S.centf, S.cnorm);
  const size_t sm = na_smem(k, d);
  switch (d) {
#define FEM_NA(DD)                                                                                    \
  case DD:                                                                                            \
    k_na_classify<DD><<<grid, kNaRows, sm, st>>>(dX, n, k, S.centf, S.cnorm, dCent, dLabels, S.part); \
    break;
    FEM_NA(2)
    FEM_NA(4)
    FEM_NA(8)
    FEM_NA(16)
    FEM_NA(32)
    FEM_NA(64)
#undef FEM_NA
  }
  k_na_final<<<1, 32, 0, st>>>(S.part, grid, n, dFit);
  const cudaError_t e = cudaGetLastError();
  if (prev != device) cudaSetDevice(prev);
  if (e != cudaSuccess) {
    set_error("fem_km_classify_noalloc: launch failed: %s", cudaGetErrorString(e));
    return FEM_ERR_CUDA;
  }
  return FEM_OK;
}
