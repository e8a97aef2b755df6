// km.cu -- Lloyd k-means iteration (NaiveKMA::ComputeMSEAndCorrect,
// Clust/KMAlgorithm.cpp:205-255) and the k-means half of the C-ABI.
//
// Assignment must equal an FP64 difference-form argmin over centroids in
// index order with strict '<' (Clust/KMAlgorithm.cpp:226-234).  Candidate
// distances are computed fast (FP32 here, BF16 tensor cores in km_tc.cu)
// together with a rigorous error bound; a row whose best candidate is not
// separated from the runner-up by the bounds is re-decided in FP64 with
// the reference's summation order.  Centroid sums are accumulated exactly
// in 64-bit fixed point (x * 2^shift is an integer for every float the
// data holds), so they are order independent; the fit uses
//   sum_i ||x_i - c_l(i)||^2 = sum_i ||x_i - g||^2
//        - 2 sum_j (c_j - g).(S_j - n_j g) + sum_j n_j ||c_j - g||^2
// with the exact cluster sums S_j and the data mean g.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "fem_internal.cuh"
#include "km_kernels.cuh"

using namespace fem;

namespace fem {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// ----------------------------------------------------------- data stats
// One pass over X for the data mean g, max |x| and sum_i ||x_i - g||^2: per
// CTA and column, S1 = sum t and S2 = sum t^2 in FP64 with t = x - c (c = the
// dataset's first row: x - c is exact in FP64 for FP32 data, and c lies inside
// the data, so S2 - S1^2 / n below does not cancel), plus max |x|.  The host
// merges the CTAs: g = c + S1 / n, sum ||x - g||^2 = sum_q (S2_q - S1_q^2 / n).
// Threads own (row group, column) pairs, so a warp reads whole rows.
__global__ void __launch_bounds__(256)
k_km_stats(const float *__restrict__ X, int64_t n, int d, int64_t rows_per_block, const float *__restrict__ c,
           double *__restrict__ s1, double *__restrict__ s2, float *__restrict__ amax) {
  __shared__ double r1[256], r2[256];
  __shared__ float rm[256];
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_block, r1e = min(n, r0 + rows_per_block);
  const bool narrow = d <= 256;
  const int groups = narrow ? 256 / d : 1;       // row groups a pass covers
  const int tid = threadIdx.x;
  float mx = 0.f;
  for (int q0 = 0; q0 < d; q0 += 256) {
    const int q = q0 + (narrow ? tid % d : tid), g = narrow ? tid / d : 0;
    const int cols = narrow ? d : min(256, d - q0);
    double a = 0.0, b = 0.0;
    if (g < groups && q < d) {
      const double cq = (double)c[q];
      for (int64_t i = r0 + g; i < r1e; i += groups) {
        const float x = X[i * d + q];
        const double t = (double)x - cq;
        a += t;
        b = fma(t, t, b);
        mx = fmaxf(mx, fabsf(x));
      }
    }
    r1[tid] = a, r2[tid] = b;
    __syncthreads();
    // column q0 + tid's row groups sit at tid + cols g: summed in group order
    if (tid < cols) {
      double sa = 0.0, sb = 0.0;
      for (int gg = 0; gg < groups; gg++) sa += r1[tid + gg * cols], sb += r2[tid + gg * cols];
      s1[(size_t)blockIdx.x * d + q0 + tid] = sa;
      s2[(size_t)blockIdx.x * d + q0 + tid] = sb;
    }
    __syncthreads();
  }
  rm[tid] = mx;
  __syncthreads();
  if (tid == 0) {
    float m = 0.f;
    for (int t = 0; t < 256; t++) m = fmaxf(m, rm[t]);
    amax[blockIdx.x] = m;
  }
}

// centroids -> float copy and norms
__global__ void k_km_prep(const double *__restrict__ cent, int K, int d, float *__restrict__ centf,
                          float *__restrict__ cnorm, __nv_bfloat16 *__restrict__ centb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K) return;
  double s = 0.0;
  for (int q = 0; q < d; q++) {
    const double c = cent[(size_t)j * d + q];
    centf[(size_t)j * d + q] = (float)c;
    if (centb) centb[(size_t)j * d + q] = __float2bfloat16_rn((float)c);
    s += c * c;
  }
  cnorm[j] = (float)sqrt(s);
}

// FP64 difference form in column order, no contraction: bit-identical to
// `for q: t = c[q] - x[q]; s += t*t;` compiled without FMA.
__device__ __forceinline__ double dist64(const double *__restrict__ c, const float *x, int d) {
  double s = 0.0;
  for (int q = 0; q < d; q++) {
    const double t = __dsub_rn(c[q], (double)x[q]);
    s = __dadd_rn(s, __dmul_rn(t, t));
  }
  return s;
}

// bound on |fp32 difference-form distance - exact distance| (x2 safety)
__device__ __forceinline__ float bound_f32(float s, float cn, int d) {
  const float u = 5.9604645e-8f;  // 2^-24
  return 2.f * ((float)(d + 4) * u * s + 2.01f * u * sqrtf(fmaxf(s, 0.f)) * cn + u * u * cn * cn) +
         1e-30f;
}

// =================================================== FP32 assignment
// One CTA per SM streams 256-row tiles; per row: FP32 difference-form
// distances to all centroids, candidate test, FP64 recheck if needed;
// then exact fixed-point accumulation of the rows into per-CTA sums.
template <int D>
__global__ void __launch_bounds__(256)
k_km_assign_f32(const float *__restrict__ X, int64_t n, int K, const float *__restrict__ centf,
                const float *__restrict__ cnorm, const double *__restrict__ cent,
                int32_t *__restrict__ labels, long long *__restrict__ accg, int *__restrict__ cntg,
                double scale, DevStatus *st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  long long *sAcc = (long long *)smem_raw;              // K x D
  float *sC = (float *)(sAcc + (size_t)K * D);          // K x D
  float *sCn = sC + (size_t)K * D;                      // K
  int *sCnt = (int *)(sCn + K);                         // K
  int *sLab = sCnt + K;                                 // 256
  float *sX = (float *)(sLab + 256);                    // 256 x (D+1)
  const int tid = threadIdx.x;
  for (int e = tid; e < K * D; e += 256) {
    sAcc[e] = 0;
    sC[e] = centf[e];
  }
  for (int j = tid; j < K; j += 256) {
    sCnt[j] = 0;
    sCn[j] = cnorm[j];
  }
  int64_t rechecks = 0;
  const int64_t ntiles = (n + 255) / 256;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t base = tile * 256;
    const int rows = (int)min((int64_t)256, n - base);
    __syncthreads();
    for (int e = tid; e < 256 * D; e += 256) {
      const int p = e / D, q = e - p * D;
      sX[p * (D + 1) + q] = (p < rows) ? X[base * D + e] : 0.f;
    }
    __syncthreads();
    int lab = -1;
    if (tid < rows) {
      float x[D];
#pragma unroll
      for (int q = 0; q < D; q++) x[q] = sX[tid * (D + 1) + q];
      float U = INFINITY, lb1 = INFINITY, lb2 = INFINITY;
      int j1 = -1;
      for (int j = 0; j < K; j++) {
        const float *c = sC + j * D;
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < D; q++) {
          const float t = x[q] - c[q];
          s = fmaf(t, t, s);
        }
        const float b = bound_f32(s, sCn[j], D);
        const float lb = s - b, ub = s + b;
        U = fminf(U, ub);
        if (lb < lb1) {
          lb2 = lb1;
          lb1 = lb;
          j1 = j;
        } else if (lb < lb2) {
          lb2 = lb;
        }
      }
      if (lb2 > U) {
        lab = j1;
      } else {
        // candidates within the bounds: decide in FP64, index order, strict <
        rechecks++;
        double best = DBL_MAX;
        for (int j = 0; j < K; j++) {
          const float *c = sC + j * D;
          float s = 0.f;
#pragma unroll
          for (int q = 0; q < D; q++) {
            const float t = x[q] - c[q];
            s = fmaf(t, t, s);
          }
          if (s - bound_f32(s, sCn[j], D) <= U) {
            const double s64 = dist64(cent + (size_t)j * D, x, D);
            if (s64 < best) {
              best = s64;
              lab = j;
            }
          }
        }
      }
      if (st->track_changes && labels[base + tid] != lab) st->changed = 1;
      labels[base + tid] = lab;
      atomicAdd(&sCnt[lab], 1);
    }
    sLab[tid] = lab;
    __syncthreads();
    // exact accumulation: warp w folds rows 32w..32w+31 into sAcc
    const int w = tid >> 5, l = tid & 31;
    for (int idx = l; idx < 32 * D; idx += 32) {
      const int p = 32 * w + idx / D, q = idx % D;
      const int lb = sLab[p];
      if (lb >= 0) {
        const long long v = __double2ll_rn((double)sX[p * (D + 1) + q] * scale);
        atomicAdd((unsigned long long *)&sAcc[lb * D + q], (unsigned long long)v);
      }
    }
  }
  __syncthreads();
  for (int e = tid; e < K * D; e += 256) accg[(size_t)blockIdx.x * K * D + e] = sAcc[e];
  for (int j = tid; j < K; j += 256) cntg[(size_t)blockIdx.x * K + j] = sCnt[j];
  if (rechecks) atomicAdd((unsigned long long *)&st->rechecked, (unsigned long long)rechecks);
}

// sums the per-CTA partials (exact), forms the new centroids and the fit terms
__global__ void k_km_final(const long long *__restrict__ accg, const int *__restrict__ cntg, int G,
                           int K, int d, double inv_scale, const double *__restrict__ cent,
                           const double *__restrict__ g, double *__restrict__ out) {
  const int j = blockIdx.x;
  __shared__ long long s_n;
  __shared__ double red[32];
  if (threadIdx.x == 0) {
    long long c = 0;
    for (int b = 0; b < G; b++) c += cntg[(size_t)b * K + j];
    s_n = c;
  }
  __syncthreads();
  const long long nj = s_n;
  double term = 0.0;
  for (int q = threadIdx.x; q < d; q += blockDim.x) {
    long long S = 0;
    for (int b = 0; b < G; b++) S += accg[((size_t)b * K + j) * d + q];
    const double sum = (double)S * inv_scale;
    out[(size_t)j * d + q] = nj > 0 ? sum * (1.0 / (double)nj) : 0.0;
    const double cg = cent[(size_t)j * d + q] - g[q];
    term += -2.0 * cg * (sum - (double)nj * g[q]) + (double)nj * cg * cg;
  }
  term = warp_sum_d(term);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = term;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) s += red[w];
    out[(size_t)K * d + j] = (double)nj;
    out[(size_t)K * d + K + j] = s;
  }
}

int km_launch_assign_f32(fem_km *h) {
  const int D = h->d, K = h->k;
  const size_t sm = (size_t)K * D * 8 + (size_t)K * D * 4 + (size_t)K * 4 + (size_t)K * 4 + 256 * 4 +
                    (size_t)256 * (D + 1) * 4;
#define FEM_KA(DD)                                                                              \
  case DD:                                                                                      \
    FEM_CUDA(allow_dyn_smem(k_km_assign_f32<DD>, sm));                                          \
    k_km_assign_f32<DD><<<h->grid, 256, sm, h->stream>>>(h->X, h->n, K, h->centf, h->cnorm,     \
                                                         h->cent, h->labels, h->acc, h->cnt,    \
                                                         ldexp(1.0, h->shift), h->dstat);       \
    break;
  switch (D) {
    FEM_KA(2)
    FEM_KA(4)
    FEM_KA(8)
    FEM_KA(16)
    FEM_KA(32)
    FEM_KA(64)
    default:
      set_error("k-means FP32 path supports d in {2,4,8,16,32,64} (got %d)", D);
      return FEM_ERR_UNSUPPORTED;
  }
#undef FEM_KA
  FEM_CUDA(cudaGetLastError());
  return FEM_OK;
}

size_t km_assign_smem(int K, int D) {
  return (size_t)K * D * 12 + (size_t)K * 8 + 1024 + (size_t)256 * (D + 1) * 4;
}

}  // namespace fem

// =============================================================== C-ABI
namespace {

int check(fem_km *h) {
  if (!h) {
    set_error("null k-means handle");
    return FEM_ERR_BAD_ARG;
  }
  return FEM_OK;
}

void free_km(fem_km *h) {
  dfree(h->X);
  dfree(h->Xb);
  dfree(h->xnorm);
  dfree(h->labels);
  dfree(h->cent);
  dfree(h->centf);
  dfree(h->centb);
  dfree(h->cnorm);
  dfree(h->acc);
  dfree(h->cnt);
  dfree(h->g);
  dfree(h->out);
  dfree(h->dstat);
  km_tc_destroy(h);
  if (h->hout) cudaFreeHost(h->hout);
  if (h->hstat) cudaFreeHost(h->hstat);
  if (h->hg) delete[] h->hg;
  h->hout = nullptr;
  h->hstat = nullptr;
  h->hg = nullptr;
  for (auto &e : h->ev)
    if (e) cudaEventDestroy(e), e = nullptr;
  if (h->stream) cudaStreamDestroy(h->stream);
  h->stream = nullptr;
}

int upload_km(fem_km *h, const float *X, int64_t ld, cudaMemcpyKind kind) {
  FEM_TRY(check(h));
  if (!X || ld < h->d) {
    set_error("bad dataset pointer or ld");
    return FEM_ERR_BAD_ARG;
  }
  const int d = h->d;
  const int64_t n = h->n;
  FEM_CUDA(cudaSetDevice(h->cfg.device));
  FEM_CUDA(cudaMemcpy2DAsync(h->X, (size_t)d * 4, X, (size_t)ld * 4, (size_t)d * 4, (size_t)n, kind,
                             h->stream));
  // data mean, max |x| -> fixed-point shift, sum ||x - g||^2, in one pass
  const int G = (int)std::min<int64_t>(4 * (int64_t)sm_count(), (n + 255) / 256);
  const int64_t rpb = (n + G - 1) / G;
  std::vector<float> c(d);
  FEM_CUDA(cudaMemcpyAsync(c.data(), h->X, (size_t)d * 4, cudaMemcpyDeviceToHost, h->stream));
  FEM_CUDA(cudaStreamSynchronize(h->stream));
  float *dc = nullptr;
  double *s1 = nullptr, *s2 = nullptr;
  float *amax = nullptr;
  FEM_TRY(dalloc(&dc, d));
  FEM_TRY(dalloc(&s1, (size_t)G * d));
  FEM_TRY(dalloc(&s2, (size_t)G * d));
  FEM_TRY(dalloc(&amax, G));
  FEM_CUDA(cudaMemcpyAsync(dc, c.data(), (size_t)d * 4, cudaMemcpyHostToDevice, h->stream));
  k_km_stats<<<G, 256, 0, h->stream>>>(h->X, n, d, rpb, dc, s1, s2, amax);
  std::vector<double> h1((size_t)G * d), h2((size_t)G * d);
  std::vector<float> hm(G);
  cudaMemcpyAsync(h1.data(), s1, h1.size() * 8, cudaMemcpyDeviceToHost, h->stream);
  cudaMemcpyAsync(h2.data(), s2, h2.size() * 8, cudaMemcpyDeviceToHost, h->stream);
  cudaMemcpyAsync(hm.data(), amax, hm.size() * 4, cudaMemcpyDeviceToHost, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  dfree(dc);
  dfree(s1);
  dfree(s2);
  dfree(amax);
  if (e != cudaSuccess) {
    set_error("dataset statistics failed: %s", cudaGetErrorString(e));
    return FEM_ERR_CUDA;
  }
  float mx = 0.f;
  for (int b = 0; b < G; b++) mx = std::max(mx, hm[b]);
  h->xg2 = 0.0;
  for (int q = 0; q < d; q++) {
    double a = 0.0, b2 = 0.0;
    for (int b = 0; b < G; b++) a += h1[(size_t)b * d + q], b2 += h2[(size_t)b * d + q];
    h->hg[q] = (double)c[q] + a / (double)n;
    h->xg2 += b2 - a * a / (double)n;
  }
  // |x| * 2^shift * n < 2^62: the per-CTA and the final int64 sums cannot overflow
  const double lg = std::log2((double)std::max(mx, 1e-30f)) + std::log2((double)n);
  h->shift = (int)std::min(40.0, std::floor(61.0 - std::ceil(lg)));
  FEM_CUDA(cudaMemcpyAsync(h->g, h->hg, d * 8, cudaMemcpyHostToDevice, h->stream));
  h->have_data = true;
  return FEM_OK;
}

}  // namespace

extern "C" {

void fem_km_config_default(fem_km_config *cfg) {
  if (!cfg) return;
  cfg->precision = FEM_PREC_MIXED;
  cfg->device = 0;
  cfg->seed = 0;
  cfg->repair = FEM_KM_REPAIR_RANDOM;
}

int fem_km_create(int d, int64_t n, int k, const fem_km_config *cfg, fem_km **out) {
  if (!out) {
    set_error("out is NULL");
    return FEM_ERR_BAD_ARG;
  }
  *out = nullptr;
  fem_km_config c;
  if (cfg)
    c = *cfg;
  else
    fem_km_config_default(&c);
  if (d < 1 || n < 1 || k < 1 || k > 1024) {
    set_error("bad sizes d=%d n=%lld k=%d", d, (long long)n, k);
    return FEM_ERR_BAD_ARG;
  }
  if (c.precision != FEM_PREC_FP32 && c.precision != FEM_PREC_MIXED) {
    set_error("k-means precision must be FEM_PREC_FP32 or FEM_PREC_MIXED");
    return FEM_ERR_BAD_ARG;
  }
  if (c.repair != FEM_KM_REPAIR_NONE && c.repair != FEM_KM_REPAIR_RANDOM && c.repair != FEM_KM_REPAIR_NEXT) {
    set_error("repair must be FEM_KM_REPAIR_NONE, FEM_KM_REPAIR_RANDOM or FEM_KM_REPAIR_NEXT");
    return FEM_ERR_BAD_ARG;
  }
  if (c.precision == FEM_PREC_FP32 && !(d == 2 || d == 4 || d == 8 || d == 16 || d == 32 || d == 64)) {
    set_error("k-means FP32 path supports d in {2,4,8,16,32,64}");
    return FEM_ERR_UNSUPPORTED;
  }
  if (c.precision == FEM_PREC_MIXED && !km_tc_supported(d, k)) {
    set_error("k-means mixed (tensor-core) path supports d = 32 and k <= 256 (got d=%d k=%d)", d, k);
    return FEM_ERR_UNSUPPORTED;
  }
  if (km_assign_smem(k, d) > 220 * 1024 && c.precision == FEM_PREC_FP32) {
    set_error("k*d too large for the shared-memory centroid table");
    return FEM_ERR_UNSUPPORTED;
  }
  FEM_TRY(select_device(c.device));
  fem_km *h = new (std::nothrow) fem_km();
  if (!h) return FEM_ERR_BAD_ARG;
  h->d = d;
  h->n = n;
  h->k = k;
  h->cfg = c;
  h->rng.seed((unsigned)c.seed);
  h->hg = new double[d];
  auto fail = [&](int st) {
    free_km(h);
    delete h;
    return st;
  };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(FEM_ERR_CUDA);
  for (auto &e : h->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(FEM_ERR_CUDA);
  h->grid = sm_count();
  int st;
  if ((st = dalloc(&h->X, (size_t)n * d)) || (st = dalloc(&h->labels, n)) ||
      (st = dalloc(&h->cent, (size_t)k * d)) || (st = dalloc(&h->centf, (size_t)k * d)) ||
      (st = dalloc(&h->cnorm, k)) || (st = dalloc(&h->acc, (size_t)h->grid * k * d)) ||
      (st = dalloc(&h->cnt, (size_t)h->grid * k)) || (st = dalloc(&h->g, d)) ||
      (st = dalloc(&h->out, (size_t)k * d + 2 * k)) || (st = dalloc(&h->dstat, 1)))
    return fail(st);
  if (cudaMallocHost(&h->hout, ((size_t)k * d + 2 * k) * 8) != cudaSuccess ||
      cudaMallocHost(&h->hstat, sizeof(DevStatus)) != cudaSuccess)
    return fail(FEM_ERR_CUDA);
  if (c.precision == FEM_PREC_MIXED && (st = km_tc_create(h))) return fail(st);
  FEM_CUDA(cudaMemsetAsync(h->labels, 0, n * 4, h->stream));
  *out = h;
  return FEM_OK;
}

void fem_km_destroy(fem_km *h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_km(h);
  delete h;
}

int fem_km_upload(fem_km *h, const float *X, int64_t ld) { return upload_km(h, X, ld, cudaMemcpyHostToDevice); }

int fem_km_upload_device(fem_km *h, const float *dX, int64_t ld) {
  return upload_km(h, dX, ld, cudaMemcpyDeviceToDevice);
}

int fem_km_init_data_structures(fem_km *h) {
  FEM_TRY(check(h));
  FEM_CUDA(cudaMemsetAsync(h->labels, 0, h->n * 4, h->stream));
  FEM_CUDA(cudaStreamSynchronize(h->stream));
  return FEM_OK;
}

int fem_km_seed(fem_km *h, uint64_t seed) {
  FEM_TRY(check(h));
  h->rng.seed((unsigned)seed);
  h->uni.reset();
  return FEM_OK;
}

int fem_km_set_rng_state(fem_km *h, const char *state) {
  FEM_TRY(check(h));
  std::mt19937_64 r;
  std::istringstream in(state ? state : "");
  if (!state || !(in >> r)) {
    set_error("fem_km_set_rng_state: not an mt19937_64 state");
    return FEM_ERR_BAD_ARG;
  }
  h->rng = r;
  h->uni.reset();
  return FEM_OK;
}

int fem_km_get_rng_state(fem_km *h, char *buf, size_t len) {
  FEM_TRY(check(h));
  std::ostringstream out;
  out << h->rng;
  const std::string t = out.str();
  if (!buf || len < t.size() + 1) {
    set_error("fem_km_get_rng_state: %zu bytes needed", t.size() + 1);
    return FEM_ERR_BAD_ARG;
  }
  std::memcpy(buf, t.c_str(), t.size() + 1);
  return FEM_OK;
}

// one Lloyd iteration (NaiveKMA::ComputeMSEAndCorrect / CorrectWithoutMSE,
// Clust/KMAlgorithm.cpp:148-255): labels, fixed-point sums, divide or repair;
// with `changed` the kernels also report whether any label moved
static int km_iterate(fem_km *h, double *centroids, double *fit, int64_t *counts, int *changed) {
  FEM_TRY(check(h));
  if (!h->have_data || !centroids) {
    set_error("k-means iteration needs an uploaded dataset and centroids");
    return FEM_ERR_STATE;
  }
  FEM_CUDA(cudaSetDevice(h->cfg.device));
  const int K = h->k, d = h->d;
  const size_t kd = (size_t)K * d;
  DevStatus z{};
  z.track_changes = changed != nullptr;
  *h->hstat = z;
  FEM_CUDA(cudaMemcpyAsync(h->dstat, h->hstat, sizeof(DevStatus), cudaMemcpyHostToDevice, h->stream));
  FEM_CUDA(cudaMemcpyAsync(h->cent, centroids, kd * 8, cudaMemcpyHostToDevice, h->stream));
  k_km_prep<<<(K + 127) / 128, 128, 0, h->stream>>>(h->cent, K, d, h->centf, h->cnorm, h->centb);
  FEM_CUDA(cudaGetLastError());
  FEM_CUDA(cudaEventRecord(h->ev[0], h->stream));
  if (h->cfg.precision == FEM_PREC_MIXED)
    FEM_TRY(km_tc_assign(h));
  else
    FEM_TRY(km_launch_assign_f32(h));
  FEM_CUDA(cudaEventRecord(h->ev[1], h->stream));
  k_km_final<<<K, 64, 0, h->stream>>>(h->acc, h->cnt, h->grid, K, d, ldexp(1.0, -h->shift), h->cent,
                                      h->g, h->out);
  FEM_CUDA(cudaGetLastError());
  FEM_CUDA(cudaEventRecord(h->ev[2], h->stream));
  FEM_CUDA(cudaMemcpyAsync(h->hout, h->out, (kd + 2 * K) * 8, cudaMemcpyDeviceToHost, h->stream));
  FEM_CUDA(cudaMemcpyAsync(h->hstat, h->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream));
  FEM_CUDA(cudaStreamSynchronize(h->stream));
  if (h->hstat->timeout) {
    set_error("a bounded device wait timed out in the tensor-core k-means kernel");
    return FEM_ERR_TIMEOUT;
  }
  float a = 0, b = 0;
  cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
  cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
  h->t_assign = a;
  h->t_update = b;
  double total = h->xg2;
  for (int j = 0; j < K; j++) total += h->hout[kd + K + j];
  if (fit) *fit = total / (double)h->n;
  // NaiveKMA: divide, or CentroidRandomRepair in index order
  for (int j = 0; j < K; j++) {
    const int64_t nj = (int64_t)h->hout[kd + j];
    if (counts) counts[j] = nj;
    if (nj > 0) {
      for (int q = 0; q < d; q++) centroids[(size_t)j * d + q] = h->hout[(size_t)j * d + q];
    } else if (h->cfg.repair != FEM_KM_REPAIR_NONE) {
      int64_t src;
      if (h->cfg.repair == FEM_KM_REPAIR_RANDOM) {
        src = (int64_t)(h->uni(h->rng) * (double)h->n);
      } else {
        src = h->next_repair;
        if (++h->next_repair == h->n) h->next_repair = 0;
      }
      std::vector<float> row(d);
      FEM_CUDA(cudaMemcpy(row.data(), h->X + src * d, d * 4, cudaMemcpyDeviceToHost));
      for (int q = 0; q < d; q++) centroids[(size_t)j * d + q] = (double)row[q];
    }
  }
  if (changed) *changed = h->hstat->changed;
  return FEM_OK;
}

int fem_km_compute_mse_and_correct(fem_km *h, double *centroids, double *fit, int64_t *counts) {
  return km_iterate(h, centroids, fit, counts, nullptr);
}

int fem_km_correct_without_mse(fem_km *h, double *centroids, int *changed) {
  if (!changed) {
    set_error("fem_km_correct_without_mse: null output");
    return FEM_ERR_BAD_ARG;
  }
  return km_iterate(h, centroids, nullptr, nullptr, changed);
}

int fem_km_run(fem_km *h, double *centroids, double min_rel, int max_iter, double *best_fit, int *iters) {
  FEM_TRY(check(h));
  double best = DBL_MAX;
  FEM_TRY(fem_km_init_data_structures(h));
  if (max_iter == 0) {
    if (best_fit) *best_fit = 0.0;
    if (iters) *iters = 0;
    return FEM_OK;
  }
  int i;
  for (i = 1;; i++) {
    double fit = 0.0;
    FEM_TRY(fem_km_compute_mse_and_correct(h, centroids, &fit, nullptr));
    const double rel = (best - fit) / best;
    if (fit < std::nextafter(fit, best))
      best = fit;
    else
      break;
    if (min_rel > 0.0 && min_rel > rel) break;
    if (max_iter > 0 && i == max_iter - 1) break;
  }
  if (best_fit) *best_fit = best;
  if (iters) *iters = i;
  return FEM_OK;
}

int fem_km_get_assignment(fem_km *h, int32_t *labels) {
  FEM_TRY(check(h));
  if (!labels) return FEM_ERR_BAD_ARG;
  FEM_CUDA(cudaMemcpyAsync(labels, h->labels, h->n * 4, cudaMemcpyDeviceToHost, h->stream));
  FEM_CUDA(cudaStreamSynchronize(h->stream));
  return FEM_OK;
}

int fem_km_stats(fem_km *h, int64_t *rechecked_rows, double *assign_ms, double *update_ms) {
  FEM_TRY(check(h));
  if (rechecked_rows) *rechecked_rows = h->hstat ? h->hstat->rechecked : 0;
  if (assign_ms) *assign_ms = h->t_assign;
  if (update_ms) *update_ms = h->t_update;
  return FEM_OK;
}

}  // extern "C"
