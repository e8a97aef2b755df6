// em_plain.cu -- CUDA-core EM sweep in FP32 or FP64 (the "plain" precision
// forms), plus the FP64 per-component factorisation shared by every form.
//
// One sweep = SimpleMatrixEM::PrecomputeDensityMatrix + MStep + the
// RegularizeCovariances / InitDensities that TrainNoCopy runs after it
// (EM2/MatrixEM.cpp:275-378, EM2/EMAlgorithm.cpp:139-191).
//
// Layout in HBM: X is n x d float rows; posteriors R are component-major
// (k x n) so every per-component pass streams contiguous memory; the
// inverse Cholesky factors are stored as W_j = L_j^-1 (lower, row-major), so
// the Mahalanobis term of point x is ||W_j (x - mu_j)||^2 (the reference
// multiplies by CholInvC = W_j^T from the right, EM2/MatrixEM.cpp:76).
#include <cfloat>
#include <cmath>
#include <cstring>

#include "fem_internal.cuh"
#include "em_kernels.cuh"
#include "em_factor.cuh"

namespace fem {

// ------------------------------------------------------------ reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// deterministic block sum (fixed shuffle tree, fixed warp order); result in thread 0
template <int NT>
__device__ double block_sum(double v, double *red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; i++) s += red[i];
  return s;
}

template <typename T> __device__ __forceinline__ T t_exp(T x);
template <> __device__ __forceinline__ float t_exp(float x) { return expf(x); }
template <> __device__ __forceinline__ double t_exp(double x) { return exp(x); }
template <typename T> __device__ __forceinline__ T t_log(T x);
template <> __device__ __forceinline__ float t_log(float x) { return logf(x); }
template <> __device__ __forceinline__ double t_log(double x) { return log(x); }

// online log-sum-exp step (max-shifted), -inf entries contribute nothing
template <typename T>
__device__ __forceinline__ void lse_push(T l, T &mx, T &se) {
  if (l > mx) {
    se = se * t_exp(mx - l) + T(1);
    mx = l;
  } else if (l > -INFINITY) {
    se += t_exp(l - mx);
  }
}

// ================================================================ E-step
// MatrixEMBase::BlockDensities + PostProcessDensityMatrix
// (EM2/MatrixEM.cpp:39-51,69-81): one thread per point, components staged
// through shared memory; l_ij is written to R, then overwritten by
// exp(l_ij - LSE_i).  D > 0: compile-time dimension with the centred point
// in registers.
template <typename T, int D>
__global__ void __launch_bounds__(128)
k_estep_plain(const float *__restrict__ X, int64_t n, int K, const T *__restrict__ mu,
              const T *__restrict__ W, const T *__restrict__ logc, T *__restrict__ R,
              double *__restrict__ part) {
  __shared__ __align__(16) T sW[D * D];
  __shared__ __align__(16) T smu[D];
  __shared__ double red[4];
  const int tid = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * 128 + tid;
  const bool valid = i < n;
  float x[D];
#pragma unroll
  for (int q = 0; q < D; q++) x[q] = valid ? X[i * D + q] : 0.f;
  T mx = -INFINITY, se = T(0);
  for (int j = 0; j < K; j++) {
    __syncthreads();
    for (int e = tid; e < D * D; e += 128) sW[e] = W[(size_t)j * D * D + e];
    if (tid < D) smu[tid] = mu[(size_t)j * D + tid];
    __syncthreads();
    T t[D];
#pragma unroll
    for (int q = 0; q < D; q++) t[q] = (T)x[q] - smu[q];
    T s = T(0);
#pragma unroll
    for (int kk = 0; kk < D; kk++) {
      T y = T(0);
#pragma unroll
      for (int m = 0; m <= kk; m++) y = fma(t[m], sW[kk * D + m], y);
      s = fma(y, y, s);
    }
    const T l = logc[j] - T(0.5) * s;
    if (valid) R[(size_t)j * n + i] = l;
    lse_push(l, mx, se);
  }
  const T lse = mx + t_log(se);
  if (valid)
    for (int j = 0; j < K; j++) {
      T *p = R + (size_t)j * n + i;
      *p = t_exp(*p - lse);
    }
  double s = block_sum<128>(valid ? (double)lse : 0.0, red);
  if (tid == 0) part[blockIdx.x] = s;
}

// runtime dimension: centred point in shared memory, factor read through L1
template <typename T>
__global__ void __launch_bounds__(64)
k_estep_plain_generic(const float *__restrict__ X, int64_t n, int d, int K,
                      const T *__restrict__ mu, const T *__restrict__ W,
                      const T *__restrict__ logc, T *__restrict__ R, double *__restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sT = (T *)smem_raw;  // 64 x (d+1)
  __shared__ double red[2];
  const int tid = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * 64 + tid;
  const bool valid = i < n;
  T *t = sT + (size_t)tid * (d + 1);
  T mx = -INFINITY, se = T(0);
  for (int j = 0; j < K; j++) {
    const T *mj = mu + (size_t)j * d;
    const T *Wj = W + (size_t)j * d * d;
    for (int q = 0; q < d; q++) t[q] = valid ? ((T)X[i * d + q] - mj[q]) : T(0);
    T s = T(0);
    for (int kk = 0; kk < d; kk++) {
      const T *wr = Wj + (size_t)kk * d;
      T y = T(0);
      for (int m = 0; m <= kk; m++) y = fma(t[m], wr[m], y);
      s = fma(y, y, s);
    }
    const T l = logc[j] - T(0.5) * s;
    if (valid) R[(size_t)j * n + i] = l;
    lse_push(l, mx, se);
  }
  const T lse = mx + t_log(se);
  if (valid)
    for (int j = 0; j < K; j++) {
      T *p = R + (size_t)j * n + i;
      *p = t_exp(*p - lse);
    }
  double s = block_sum<64>(valid ? (double)lse : 0.0, red);
  if (tid == 0) part[blockIdx.x] = s;
}

// register-tiled form for d > 64: a CTA of 256 threads takes P = 32 PT
// points.  Per component the centred points are staged once, transposed
// (sT[m][p], pitch P + 1), and L^-1 is streamed through 64 x 64 chunks
// (sW[m][o], pitch 68) up to the diagonal: output chunk o0 needs columns
// m < o0 + 64 only (the factor's upper triangle is stored as zeros, so the
// diagonal chunk needs no mask).  Thread (tp, to) = (tid / 8, tid % 8)
// holds y for points tp + 32 i (i < PT) and outputs o0 + 8 to + (0..7): per
// column m, PT broadcast loads of t and one 8-wide load of W feed 8 PT FMAs.
// s = ||y||^2 is summed per thread over its outputs, then over the 8 threads
// of a point group by a fixed shuffle tree (run-to-run reproducible).
constexpr int kETileOC = 64;              // outputs per chunk
constexpr int kETileMC = 64;              // factor columns per chunk
constexpr int kETileWP = kETileOC + 4;    // sW pitch (16-byte rows)
constexpr size_t kMaxDynSmem = 232448;    // opt-in shared memory per CTA (227 KB)

// 8 consecutive elements from a 16-byte-aligned shared-memory address
__device__ __forceinline__ void load8(const float *p, float (&v)[8]) {
  const float4 a = reinterpret_cast<const float4 *>(p)[0], b = reinterpret_cast<const float4 *>(p)[1];
  v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
}
__device__ __forceinline__ void load8(const double *p, double (&v)[8]) {
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const double2 a = reinterpret_cast<const double2 *>(p)[q];
    v[2 * q] = a.x, v[2 * q + 1] = a.y;
  }
}

template <typename T, int PT>
constexpr size_t estep_tiled_smem(int d) {
  return ((size_t)((d + 63) & ~63) * (32 * PT + 1) + (size_t)kETileMC * kETileWP + 32 * PT) * sizeof(T);
}

template <typename T, int PT>
__global__ void __launch_bounds__(256)
k_estep_plain_tiled(const float *__restrict__ X, int64_t n, int d, int K, const T *__restrict__ mu,
                    const T *__restrict__ W, const T *__restrict__ logc, T *__restrict__ R,
                    double *__restrict__ part) {
  constexpr int P = 32 * PT, TP = P + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int dpad = (d + 63) & ~63;
  T *sW = (T *)smem_raw;                       // kETileMC x kETileWP (first: 16-byte aligned rows)
  T *sT = sW + kETileMC * kETileWP;            // dpad x TP
  T *sLse = sT + (size_t)dpad * TP;            // P
  __shared__ double red[8];
  const int tid = threadIdx.x, to = tid & 7, tp = tid >> 3;
  const int64_t i0 = (int64_t)blockIdx.x * P;
  T mx[PT], se[PT];
#pragma unroll
  for (int i = 0; i < PT; i++) mx[i] = -INFINITY, se[i] = T(0);
  for (int j = 0; j < K; j++) {
    const T *mj = mu + (size_t)j * d;
    const T *Wj = W + (size_t)j * d * d;
    __syncthreads();                           // the previous component's reads of sT are done
    // coalesced rows of X (column fastest); pitch TP puts consecutive
    // columns of one point in consecutive banks
    for (int e = tid; e < P * dpad; e += 256) {
      const int p = e / dpad, m = e - p * dpad;
      T t = T(0);
      if (m < d && i0 + p < n) t = (T)X[(i0 + p) * d + m] - mj[m];
      sT[(size_t)m * TP + p] = t;
    }
    T s[PT];
#pragma unroll
    for (int i = 0; i < PT; i++) s[i] = T(0);
    for (int o0 = 0; o0 < dpad; o0 += kETileOC) {
      T y[PT][8];
#pragma unroll
      for (int i = 0; i < PT; i++)
#pragma unroll
        for (int o = 0; o < 8; o++) y[i][o] = T(0);
      for (int m0 = 0; m0 <= o0; m0 += kETileMC) {
        __syncthreads();                       // sW free (and sT staged, on the first chunk)
        for (int e = tid; e < kETileOC * kETileMC; e += 256) {
          const int o = e / kETileMC, m = e - o * kETileMC;
          const int go = o0 + o, gm = m0 + m;
          sW[m * kETileWP + o] = (go < d && gm < d) ? Wj[(size_t)go * d + gm] : T(0);
        }
        __syncthreads();
        const T *tcol = sT + (size_t)m0 * TP + tp;
        const T *wrow = sW + to * 8;
#pragma unroll 4
        for (int m = 0; m < kETileMC; m++) {
          T tv[PT], wv[8];
#pragma unroll
          for (int i = 0; i < PT; i++) tv[i] = tcol[(size_t)m * TP + 32 * i];
          load8(wrow + m * kETileWP, wv);
#pragma unroll
          for (int i = 0; i < PT; i++)
#pragma unroll
            for (int o = 0; o < 8; o++) y[i][o] = fma(tv[i], wv[o], y[i][o]);
        }
      }
#pragma unroll
      for (int i = 0; i < PT; i++)
#pragma unroll
        for (int o = 0; o < 8; o++) s[i] = fma(y[i][o], y[i][o], s[i]);
    }
    // the 8 threads of a point group are 8 consecutive lanes
#pragma unroll
    for (int i = 0; i < PT; i++) {
      s[i] += __shfl_xor_sync(0xffffffffu, s[i], 1);
      s[i] += __shfl_xor_sync(0xffffffffu, s[i], 2);
      s[i] += __shfl_xor_sync(0xffffffffu, s[i], 4);
    }
    if (to == 0) {
      const T lc = logc[j];
#pragma unroll
      for (int i = 0; i < PT; i++) {
        const int64_t pi = i0 + tp + 32 * i;
        const T l = lc - T(0.5) * s[i];
        if (pi < n) R[(size_t)j * n + pi] = l;
        lse_push(l, mx[i], se[i]);
      }
    }
  }
  double v = 0.0;
  if (to == 0)
#pragma unroll
    for (int i = 0; i < PT; i++) {
      const T lse = mx[i] + t_log(se[i]);
      sLse[tp + 32 * i] = lse;
      if (i0 + tp + 32 * i < n) v += (double)lse;
    }
  __syncthreads();                             // sLse and every l_ij of this CTA written
  for (int e = tid; e < K * P; e += 256) {
    const int j = e / P, p = e - j * P;
    if (i0 + p < n) {
      T *q = R + (size_t)j * n + i0 + p;
      *q = t_exp(*q - sLse[p]);
    }
  }
  const double ls = block_sum<256>(v, red);
  if (tid == 0) part[blockIdx.x] = ls;
}

// single-block deterministic sum of the per-block log-likelihood partials
__global__ void __launch_bounds__(1024) k_reduce_logl(const double *part, int64_t np, DevStatus *st) {
  __shared__ double red[32];
  double v = 0.0;
  for (int64_t b = threadIdx.x; b < np; b += 1024) v += part[b];
  double s = block_sum<1024>(v, red);
  if (threadIdx.x == 0) st->logl = s;
}

// ======================================================= M-step: means
// SimpleMatrixEM::doMStep means part (EM2/MatrixEM.cpp:319-343):
// PosteriorSum_j = sum_i r_ij and MeanSums_j = sum_i r_ij x_i per block of
// rows; each thread owns (component, C-column chunk) units.  The last chunk
// of a row may be partial (C does not divide d): its lanes past column d
// read staged values of the next row (or the padding after the last one)
// and are never written out.
constexpr int kMeanTP = 32;

template <typename T, int C, int UPT>
__global__ void __launch_bounds__(256)
k_means_plain(const float *__restrict__ X, int64_t n, int d, int K, const T *__restrict__ R,
              double *__restrict__ part, int64_t rows_per_block) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *sX = (float *)smem_raw;                       // TP x d, then C floats of padding
  T *sR = (T *)(sX + kMeanTP * d + C);                 // K x (TP+1)
  const int tid = threadIdx.x;
  const int nch = (d + C - 1) / C, units = K * nch;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
  const int64_t r1 = min(n, r0 + rows_per_block);
  T acc[UPT][C], acc1[UPT];
  double dacc[UPT][C], dacc1[UPT];
#pragma unroll
  for (int u = 0; u < UPT; u++) {
    acc1[u] = T(0);
    dacc1[u] = 0.0;
#pragma unroll
    for (int a = 0; a < C; a++) acc[u][a] = T(0), dacc[u][a] = 0.0;
  }
  int tiles = 0;
  for (int64_t t0 = r0; t0 < r1; t0 += kMeanTP) {
    const int tp = (int)min((int64_t)kMeanTP, r1 - t0);
    __syncthreads();
    for (int e = tid; e < kMeanTP * d; e += 256) {
      int p = e / d;
      sX[e] = (p < tp) ? X[(t0 + p) * d + (e - p * d)] : 0.f;
    }
    for (int e = tid; e < K * kMeanTP; e += 256) {
      int j = e / kMeanTP, p = e - j * kMeanTP;
      sR[j * (kMeanTP + 1) + p] = (p < tp) ? R[(size_t)j * n + t0 + p] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < UPT; u++) {
      const int unit = tid + u * 256;
      if (unit < units) {
        const int j = unit / nch, c = unit - j * nch;
        const T *rr = sR + j * (kMeanTP + 1);
        const float *xx = sX + c * C;
        for (int p = 0; p < kMeanTP; p++) {
          const T r = rr[p];
          acc1[u] += r;
#pragma unroll
          for (int a = 0; a < C; a++) acc[u][a] = fma(r, (T)xx[p * d + a], acc[u][a]);
        }
      }
    }
    // flush the short-range accumulators into FP64 every 16 tiles
    if (++tiles == 16 || t0 + kMeanTP >= r1) {
      tiles = 0;
#pragma unroll
      for (int u = 0; u < UPT; u++) {
        dacc1[u] += (double)acc1[u];
        acc1[u] = T(0);
#pragma unroll
        for (int a = 0; a < C; a++) {
          dacc[u][a] += (double)acc[u][a];
          acc[u][a] = T(0);
        }
      }
    }
  }
#pragma unroll
  for (int u = 0; u < UPT; u++) {
    const int unit = tid + u * 256;
    if (unit < units) {
      const int j = unit / nch, c = unit - j * nch;
      double *o = part + ((size_t)blockIdx.x * K + j) * (d + 1);
      if (c == 0) o[0] = dacc1[u];
#pragma unroll
      for (int a = 0; a < C; a++)
        if (c * C + a < d) o[1 + c * C + a] = dacc[u][a];
    }
  }
}

// PosteriorSum, Means = MeanSums / PosteriorSum, Probs = PosteriorSum / N
// (EM2/MatrixEM.cpp:341-343,375); one block per component, blocks summed in order
template <typename T>
__global__ void k_final_means(const double *__restrict__ part, int G, int K, int d, int64_t n,
                              double *__restrict__ mu, double *__restrict__ pi,
                              double *__restrict__ psum, T *__restrict__ muT) {
  const int j = blockIdx.x;
  __shared__ double s1;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int g = 0; g < G; g++) s += part[((size_t)g * K + j) * (d + 1)];
    s1 = s;
    psum[j] = s;
    pi[j] = s / (double)n;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < d; q += blockDim.x) {
    double s = 0.0;
    for (int g = 0; g < G; g++) s += part[((size_t)g * K + j) * (d + 1) + 1 + q];
    const double m = s / s1;
    mu[(size_t)j * d + q] = m;
    muT[(size_t)j * d + q] = (T)m;
  }
}

// ================================================== M-step: covariances
// MatrixEMBase::ComputeWeightedTempDataset + BlockCovariances
// (EM2/MatrixEM.cpp:53-67,90-99): z = sqrt(r_ij) (x_i - mu_j), CovSum_j +=
// z z^T over the upper block triangle.  Each thread owns one TB x TB block
// of one component; a CTA owns 256 consecutive (component, block) units.
constexpr int kCovTP = 32;
constexpr int kCovFlushTiles = 64;   // FP32 sums span at most 64 tiles (2048 rows)

// posterior (component j, point i): typed component-major array, or the
// mixed path's FP16 hi + lo pair
template <typename T>
struct PostTyped {
  const T *R;
  int64_t pitch;
  __device__ T operator()(int j, int64_t i) const { return R[(size_t)j * pitch + i]; }
};
struct PostHiLo {
  const __half *Rh, *Rl;
  int64_t pitch;
  __device__ float operator()(int j, int64_t i) const {
    const size_t o = (size_t)j * pitch + i;
    return __half2float(Rh[o]) + __half2float(Rl[o]);
  }
};

template <typename T, int TB, class Src>
__global__ void __launch_bounds__(256)
k_cov_plain(const float *__restrict__ X, int64_t n, int d, int K, Src R, const T *__restrict__ mu, int mu_ld,
            double *__restrict__ part, int nb, int nblk, int64_t rows_per_chunk, int upc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sZ = (T *)smem_raw;  // CJ x TP x d
  const int tid = threadIdx.x;
  // this CTA's upc (<= 256, a multiple of 32) units; the components they
  // span are staged, so small d with many components takes fewer units
  const int u0 = blockIdx.x * upc;
  const int j_lo = u0 / nblk;
  const int j_hi = min(K - 1, (u0 + upc - 1) / nblk);
  const int CJ = j_hi - j_lo + 1;
  T *sSr = sZ + (size_t)CJ * kCovTP * d;  // CJ x TP: sqrt(r), once per point and component
  const int unit = u0 + tid;
  const bool valid = tid < upc && unit < K * nblk;
  int j = 0, bi = 0, bj = 0;
  if (valid) {
    j = unit / nblk;
    int b = unit - j * nblk;
    // upper-triangular enumeration of nb x nb blocks: row bi has nb - bi blocks
    while (b >= nb - bi) {
      b -= nb - bi;
      bi++;
    }
    bj = bi + b;
  }
  const int64_t c0 = (int64_t)blockIdx.y * rows_per_chunk;
  const int64_t c1 = min(n, c0 + rows_per_chunk);
  T acc[TB][TB];
#pragma unroll
  for (int a = 0; a < TB; a++)
#pragma unroll
    for (int b = 0; b < TB; b++) acc[a][b] = T(0);
  const int cj = j - j_lo;
  // this thread's FP64 partial block (owned by it alone): the FP32 sums are
  // added into it every kCovFlushTiles tiles, so FP32 never sums more than
  // 2048 rows (ill-conditioned covariances stay positive definite)
  double *o = valid ? part + (((size_t)blockIdx.y * K + j) * nblk + (unit - j * nblk)) * (TB * TB) : nullptr;
  if (valid)
#pragma unroll
    for (int e = 0; e < TB * TB; e++) o[e] = 0.0;
  int tiles = 0;
  for (int64_t t0 = c0; t0 < c1; t0 += kCovTP) {
    const int tp = (int)min((int64_t)kCovTP, c1 - t0);
    __syncthreads();
    for (int e = tid; e < CJ * kCovTP; e += 256) {
      const int jj = e / kCovTP, p = e - jj * kCovTP;
      sSr[e] = p < tp ? sqrt((T)R(j_lo + jj, t0 + p)) : T(0);
    }
    __syncthreads();
    const int tot = CJ * kCovTP * d;
    for (int e = tid; e < tot; e += 256) {
      const int jj = e / (kCovTP * d);
      const int rem = e - jj * kCovTP * d;
      const int p = rem / d, a = rem - p * d;
      T z = T(0);
      if (p < tp) {
        const int64_t row = t0 + p;
        z = sSr[jj * kCovTP + p] * ((T)X[row * d + a] - mu[(size_t)(j_lo + jj) * mu_ld + a]);
      }
      sZ[e] = z;
    }
    __syncthreads();
    if (valid) {
      const T *zb = sZ + (size_t)cj * kCovTP * d;
      for (int p = 0; p < kCovTP; p++) {
        const T *zr = zb + p * d;
        T va[TB], vb[TB];
#pragma unroll
        for (int a = 0; a < TB; a++) va[a] = zr[bi * TB + a];
#pragma unroll
        for (int b = 0; b < TB; b++) vb[b] = zr[bj * TB + b];
#pragma unroll
        for (int a = 0; a < TB; a++)
#pragma unroll
          for (int b = 0; b < TB; b++) acc[a][b] = fma(va[a], vb[b], acc[a][b]);
      }
      if (++tiles == kCovFlushTiles || t0 + kCovTP >= c1) {
        tiles = 0;
#pragma unroll
        for (int a = 0; a < TB; a++)
#pragma unroll
          for (int b = 0; b < TB; b++) o[a * TB + b] += (double)acc[a][b], acc[a][b] = T(0);
      }
    }
  }
}

// Covs_j = CovSum_j / PosteriorSum_j, upper mirrored to lower (EM2/MatrixEM.cpp:370-373)
__global__ void k_final_cov(const double *__restrict__ part, int chunks, int K, int d, int nb,
                            int nblk, int TB, const double *__restrict__ psum,
                            double *__restrict__ sigma) {
  const int j = blockIdx.x;
  const double inv = 1.0 / psum[j];
  double *S = sigma + (size_t)j * d * d;
  const int per = TB * TB;
  for (int e = threadIdx.x; e < nblk * per; e += blockDim.x) {
    int b = e / per, w = e - b * per;
    int bi = 0, bb = b;
    while (bb >= nb - bi) {
      bb -= nb - bi;
      bi++;
    }
    const int bj = bi + bb;
    const int a = bi * TB + w / TB, c = bj * TB + (w % TB);
    if (a > c) continue;  // lower half of a diagonal block
    double s = 0.0;
    for (int ch = 0; ch < chunks; ch++) s += part[(((size_t)ch * K + j) * nblk + b) * per + w];
    s *= inv;
    S[(size_t)a * d + c] = s;
    S[(size_t)c * d + a] = s;
  }
}

// ======================================================= factorisation
// EMAlgorithm::RegularizeCovariances + NormalDensity::Init + CalcLogCoeffs
// (EM2/EMAlgorithm.cpp:237-244, EM2/NormalDensity.cpp:43-65,
// EM2/MatrixEM.cpp:83-87) in FP64, one CTA per component: symmetric copy of
// the lower triangle, right-looking Cholesky (a pivot <= 0 fails, as in
// Eigen's LLT), log det = 2 sum log L_ii, W = L^-1 by column substitution,
// log coefficient log pi_j - d/2 log 2pi - 1/2 log det, and an upper bound
// of the condition number (block_cond_bound) folded into st->cond_bound.
// From d = kFactorBlockedD on, the Cholesky and L^-1 run blocked through
// factor_smem_bytes(d) of dynamic shared memory (block_cholesky_panels,
// block_lower_inverse_rows: the same bits, 7.8 -> 3.3 ms for 64 components at
// d = 256); below it the unblocked forms are faster (0.24 against 0.26 ms at
// d = 64).
template <typename T>
__global__ void __launch_bounds__(kFactorThreads)
k_factor(int K, int d, double reg, int regularize, double *__restrict__ sigma,
         const double *__restrict__ pi, const double *__restrict__ mu, double *__restrict__ work,
         double *__restrict__ linv, double *__restrict__ logdet, double *__restrict__ logc,
         T *__restrict__ muT, T *__restrict__ linvT, T *__restrict__ logcT, DevStatus *st) {
  const int j = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  double *S = sigma + (size_t)j * d * d;
  double *A = work + (size_t)j * d * d;
  double *Wi = linv + (size_t)j * d * d;
  extern __shared__ double fsm[];
  if (regularize && reg != 0.0) block_regularize(S, d, reg);
  const bool blocked = d >= kFactorBlockedD;
  if (!(blocked ? block_cholesky_panels(S, d, A, fsm) : block_cholesky(S, d, A))) {
    if (tid == 0) atomicMin(&st->chol_failed, j);
    return;
  }
  if (blocked)
    block_lower_inverse_rows(A, d, Wi, fsm);
  else
    block_lower_inverse(A, d, Wi);
  const double ld = block_chol_logdet(A, d);
  const double cb = block_cond_bound(S, Wi, d);
  if (tid == 0) {
    // non-negative doubles order like their bit patterns
    atomicMax(reinterpret_cast<unsigned long long *>(&st->cond_bound), (unsigned long long)__double_as_longlong(cb));
    logdet[j] = ld;
    const double lc = log(pi[j]) - 0.5 * (double)d * log(2.0 * M_PI) - 0.5 * ld;
    logc[j] = lc;
    logcT[j] = (T)lc;
  }
  for (int e = tid; e < d * d; e += nt) linvT[(size_t)j * d * d + e] = (T)Wi[e];
  for (int q = tid; q < d; q += nt) muT[(size_t)j * d + q] = (T)mu[(size_t)j * d + q];
}

// =========================================================== launchers
template <typename T>
static int estep_plain_t(fem_em *h) {
  const int64_t n = h->n;
  const int d = h->d, K = h->k;
  const T *mu = (const T *)h->muT, *W = (const T *)h->linvT, *lc = (const T *)h->logcT;
  T *R = (T *)h->R;
  cudaStream_t s = h->stream;
  int64_t nb;
#define FEM_EPL(DD)                                                                        \
  case DD:                                                                                 \
    nb = (n + 127) / 128;                                                                  \
    k_estep_plain<T, DD><<<(unsigned)nb, 128, 0, s>>>(h->X, n, K, mu, W, lc, R, h->logl_part); \
    break;
  switch (d) {
    FEM_EPL(4)
    FEM_EPL(8)
    FEM_EPL(16)
    FEM_EPL(32)
    FEM_EPL(64)
    default: {
      constexpr int PT = sizeof(T) == 4 ? 4 : 2;   // 128 FP32 or 64 FP64 points per CTA
      const size_t smt = estep_tiled_smem<T, PT>(d);
      if (d > 64 && smt <= kMaxDynSmem) {
        nb = (n + 32 * PT - 1) / (32 * PT);
        FEM_CUDA(allow_dyn_smem(k_estep_plain_tiled<T, PT>, smt));
        k_estep_plain_tiled<T, PT><<<(unsigned)nb, 256, smt, s>>>(h->X, n, d, K, mu, W, lc, R, h->logl_part);
      } else {
        nb = (n + 63) / 64;
        size_t sm = (size_t)64 * (d + 1) * sizeof(T);
        FEM_CUDA(allow_dyn_smem(k_estep_plain_generic<T>, sm));
        k_estep_plain_generic<T><<<(unsigned)nb, 64, sm, s>>>(h->X, n, d, K, mu, W, lc, R,
                                                              h->logl_part);
      }
    }
  }
#undef FEM_EPL
  FEM_CUDA(cudaGetLastError());
  k_reduce_logl<<<1, 1024, 0, s>>>(h->logl_part, nb, h->dstat);
  FEM_CUDA(cudaGetLastError());
  h->launches += 2;
  return FEM_OK;
}

int em_plain_estep(fem_em *h) {
  return h->cfg.precision == FEM_PREC_FP64 ? estep_plain_t<double>(h) : estep_plain_t<float>(h);
}

int64_t em_plain_logl_blocks(int64_t n, int d) {
  switch (d) {
    case 4: case 8: case 16: case 32: case 64: return (n + 127) / 128;
    default: return (n + 63) / 64;
  }
}

// tiles of TB x TB covariance entries; TB divides d, so no tile reaches past
// the last dimension
void cov_geometry(int d, int *TB, int *nb, int *nblk) {
  *TB = d % 8 == 0 ? 8 : (d % 4 == 0 ? 4 : (d % 2 == 0 ? 2 : 1));
  *nb = d / *TB;
  *nblk = (*nb) * (*nb + 1) / 2;
}

template <typename T, int C>
static int launch_means(fem_em *h, int upt, int64_t rpb, size_t sm) {
  const T *R = (const T *)h->R;
#define FEM_ML(U)                                                                          \
  if (upt == U) {                                                                          \
    FEM_CUDA(allow_dyn_smem(k_means_plain<T, C, U>, sm));                                  \
    k_means_plain<T, C, U><<<h->mgrid, 256, sm, h->stream>>>(h->X, h->n, h->d, h->k, R,     \
                                                             h->mpart, rpb);               \
    return FEM_OK;                                                                         \
  }
  FEM_ML(1)
  FEM_ML(2)
  FEM_ML(4)
#undef FEM_ML
  set_error("means kernel: %d units per thread unsupported", upt);
  return FEM_ERR_UNSUPPORTED;
}

template <typename T, int TB, class Src>
static int launch_cov(fem_em *h, int nb, int nblk, int64_t rpc, Src src, const T *mu, int mu_ld) {
  const int units = h->k * nblk;
  // z tiles + sqrt(r) of the components that upc consecutive units span
  auto smem = [&](int upc) {
    return (size_t)min((upc - 1) / nblk + 2, h->k) * kCovTP * (h->d + 1) * sizeof(T);
  };
  int upc = 256;
  while (upc > 32 && smem(upc) > kMaxDynSmem) upc -= 32;
  if (smem(upc) > kMaxDynSmem) {
    set_error("covariance tiles of d = %d need %zu bytes of shared memory", h->d, smem(upc));
    return FEM_ERR_UNSUPPORTED;
  }
  const size_t sm = smem(upc);
  const int gx = (units + upc - 1) / upc;
  FEM_CUDA(allow_dyn_smem(k_cov_plain<T, TB, Src>, sm));
  dim3 grid(gx, h->cchunks);
  k_cov_plain<T, TB, Src><<<grid, 256, sm, h->stream>>>(h->X, h->n, h->d, h->k, src, mu, mu_ld, h->cpart, nb,
                                                        nblk, rpc, upc);
  return FEM_OK;
}

// the covariance pass for any posterior source: partials + FP64 finalisation
template <typename T, class Src>
static int cov_pass(fem_em *h, Src src, const T *mu, int mu_ld) {
  const int d = h->d, K = h->k;
  int TB, nb, nblk, st;
  cov_geometry(d, &TB, &nb, &nblk);
  const int64_t rpc = (h->n + h->cchunks - 1) / h->cchunks;
  if (TB == 8)
    st = launch_cov<T, 8>(h, nb, nblk, rpc, src, mu, mu_ld);
  else if (TB == 4)
    st = launch_cov<T, 4>(h, nb, nblk, rpc, src, mu, mu_ld);
  else if (TB == 2)
    st = launch_cov<T, 2>(h, nb, nblk, rpc, src, mu, mu_ld);
  else
    st = launch_cov<T, 1>(h, nb, nblk, rpc, src, mu, mu_ld);
  FEM_TRY(st);
  FEM_CUDA(cudaGetLastError());
  k_final_cov<<<K, 256, 0, h->stream>>>(h->cpart, h->cchunks, K, d, nb, nblk, TB, h->psum, h->sigma);
  FEM_CUDA(cudaGetLastError());
  return FEM_OK;
}

int em_cov_hilo(fem_em *h, const __half *Rh, const __half *Rl, int64_t pitch, const float *muf, int mu_ld) {
  FEM_TRY((cov_pass<float, PostHiLo>(h, PostHiLo{Rh, Rl, pitch}, muf, mu_ld)));
  h->launches += 2;
  return FEM_OK;
}

template <typename T>
static int mstep_plain_t(fem_em *h) {
  const int d = h->d, K = h->k;
  const int64_t n = h->n;
  // column chunk: the smallest of 4, 8, 16 covering d, else 32 (any d)
  const int C = d <= 4 ? 4 : (d <= 8 ? 8 : (d <= 16 ? 16 : 32));
  const int units = K * ((d + C - 1) / C);
  const int upt = units <= 256 ? 1 : (units <= 512 ? 2 : (units <= 1024 ? 4 : 0));
  if (upt == 0) {
    set_error("plain M-step: k*d too large (k=%d d=%d)", K, d);
    return FEM_ERR_UNSUPPORTED;
  }
  const int64_t rpb = (n + h->mgrid - 1) / h->mgrid;
  size_t sm = ((size_t)kMeanTP * d + C) * sizeof(float) + (size_t)K * (kMeanTP + 1) * sizeof(T);
  int st;
  switch (C) {
    case 4: st = launch_means<T, 4>(h, upt, rpb, sm); break;
    case 8: st = launch_means<T, 8>(h, upt, rpb, sm); break;
    case 16: st = launch_means<T, 16>(h, upt, rpb, sm); break;
    case 32: st = launch_means<T, 32>(h, upt, rpb, sm); break;
    default: set_error("unsupported d=%d", d); return FEM_ERR_UNSUPPORTED;
  }
  FEM_TRY(st);
  FEM_CUDA(cudaGetLastError());
  k_final_means<T><<<K, 128, 0, h->stream>>>(h->mpart, h->mgrid, K, d, n, h->mu, h->pi, h->psum,
                                             (T *)h->muT);
  FEM_CUDA(cudaGetLastError());
  FEM_TRY((cov_pass<T, PostTyped<T>>(h, PostTyped<T>{(const T *)h->R, n}, (const T *)h->muT, d)));
  h->launches += 4;
  return FEM_OK;
}

int em_plain_mstep(fem_em *h) {
  return h->cfg.precision == FEM_PREC_FP64 ? mstep_plain_t<double>(h) : mstep_plain_t<float>(h);
}

constexpr size_t kJacobiSmem = 96 * 1024;

// NormalDensity::ComputeConditionNumber (EM2/NormalDensity.cpp:67-71), one
// CTA per component on a symmetric copy of Sigma_j (block_jacobi_cond); the
// largest cond_j is folded into *out (non-negative doubles order like their bits).
__global__ void __launch_bounds__(256)
k_cond_jacobi(const double *__restrict__ sigma, int d, double *__restrict__ work, unsigned long long *out) {
  extern __shared__ double smem_jac[];
  const int j = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  // the matrix lives in shared memory when it fits (d <= 110), else in `work`
  double *A = (size_t)d * d * sizeof(double) <= kJacobiSmem ? smem_jac : work + (size_t)j * d * d;
  const double *S = sigma + (size_t)j * d * d;
  for (int e = tid; e < d * d; e += nt) {
    const int r = e / d, c = e - r * d;
    A[e] = (c <= r) ? S[e] : S[(size_t)c * d + r];
  }
  __syncthreads();
  const double cond = block_jacobi_cond(A, d);
  if (tid == 0) atomicMax(out, (unsigned long long)__double_as_longlong(cond));
}

int em_max_cond(fem_em *h, double *cond) {
  if (h->d > 256) {
    set_error("condition check supports d <= 256 (got %d)", h->d);
    return FEM_ERR_UNSUPPORTED;
  }
  unsigned long long *dout = nullptr;
  FEM_TRY(dalloc(&dout, 1));
  FEM_CUDA(cudaMemsetAsync(dout, 0, sizeof(unsigned long long), h->stream));
  const size_t sm = (size_t)h->d * h->d * sizeof(double) <= kJacobiSmem ? (size_t)h->d * h->d * sizeof(double) : 0;
  FEM_CUDA(allow_dyn_smem(k_cond_jacobi, sm));
  k_cond_jacobi<<<h->k, 256, sm, h->stream>>>(h->sigma, h->d, h->work, dout);
  cudaError_t e = cudaGetLastError();
  unsigned long long bits = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, dout, sizeof(bits), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  dfree(dout);
  if (e != cudaSuccess) {
    set_error("condition-number kernel failed: %s", cudaGetErrorString(e));
    return FEM_ERR_CUDA;
  }
  std::memcpy(cond, &bits, sizeof(double));
  h->launches += 1;
  return FEM_OK;
}

int em_factor(fem_em *h, bool regularize) {
  const int K = h->k, d = h->d;
  const size_t sm = d >= kFactorBlockedD ? factor_smem_bytes(d) : 0;
  if (h->cfg.precision == FEM_PREC_FP64) {
    FEM_CUDA(allow_dyn_smem(k_factor<double>, sm));
    k_factor<double><<<K, kFactorThreads, sm, h->stream>>>(K, d, h->cfg.reg_coef, regularize, h->sigma, h->pi,
                                               h->mu, h->work, h->linv, h->logdet, h->logc,
                                               (double *)h->muT, (double *)h->linvT,
                                               (double *)h->logcT, h->dstat);
  } else {
    FEM_CUDA(allow_dyn_smem(k_factor<float>, sm));
    k_factor<float><<<K, kFactorThreads, sm, h->stream>>>(K, d, h->cfg.reg_coef, regularize, h->sigma, h->pi,
                                              h->mu, h->work, h->linv, h->logdet, h->logc,
                                              (float *)h->muT, (float *)h->linvT,
                                              (float *)h->logcT, h->dstat);
  }
  FEM_CUDA(cudaGetLastError());
  h->launches += 1;
  return FEM_OK;
}

// ------------------------------------------------ posteriors read-back
template <typename T>
__global__ void k_post_rows(const T *__restrict__ R, int64_t n, int K, int64_t r0, int64_t rows,
                            double *__restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * K) return;
  const int64_t i = e / K;
  const int j = (int)(e - i * K);
  out[e] = (double)R[(size_t)j * n + r0 + i];
}

// EMAlgorithm::RetrieveClasses: first index of the largest posterior
template <typename T>
__global__ void k_classes(const T *__restrict__ R, int64_t n, int K, int32_t *__restrict__ cls) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double best = -1.0;
  int bj = -1;
  for (int j = 0; j < K; j++) {
    const double v = (double)R[(size_t)j * n + i];
    if (v > best) {
      best = v;
      bj = j;
    }
  }
  cls[i] = bj;
}

int em_post_rows(fem_em *h, int64_t r0, int64_t rows, double *dout) {
  const int64_t tot = rows * h->k;
  const unsigned nb = (unsigned)((tot + 255) / 256);
  if (h->cfg.precision == FEM_PREC_FP64)
    k_post_rows<double><<<nb, 256, 0, h->stream>>>((const double *)h->R, h->n, h->k, r0, rows, dout);
  else
    k_post_rows<float><<<nb, 256, 0, h->stream>>>((const float *)h->R, h->n, h->k, r0, rows, dout);
  FEM_CUDA(cudaGetLastError());
  return FEM_OK;
}

int em_classes(fem_em *h, int32_t *dcls) {
  const unsigned nb = (unsigned)((h->n + 255) / 256);
  if (h->cfg.precision == FEM_PREC_FP64)
    k_classes<double><<<nb, 256, 0, h->stream>>>((const double *)h->R, h->n, h->k, dcls);
  else
    k_classes<float><<<nb, 256, 0, h->stream>>>((const float *)h->R, h->n, h->k, dcls);
  FEM_CUDA(cudaGetLastError());
  return FEM_OK;
}

}  // namespace fem
