// em_batch.cu -- many independent mixture fits trained together on one GPU.
//
// Each fit follows EMAlgorithm::TrainNoCopy (EM2/EMAlgorithm.cpp:139-191)
// with the SimpleMatrixEM sweep (EM2/MatrixEM.cpp:275-378) on its own data,
// parameters, convergence test and failure status, exactly as one
// fem_em_train call would; what changes is the schedule.  Every kernel of a
// sweep covers all fits that are still active, so a batch of small fits costs
// a handful of launches per sweep rather than a handful per fit, and the host
// waits on the device only every kBatchSyncEvery sweeps (to stop early once
// every fit has converged or failed).
//
// Precision: FP32 on CUDA cores for the E-step, means and covariance sums
// (the fem_em FP32 form); FP64 for the per-item partial sums, the reductions,
// the Cholesky factors, log-determinants and LogL.
//
// Shapes: d <= 32, k <= 64, n < 2^31 per fit.  A fit's dimension class
// D in {4, 8, 16, 32} is the next power of two >= max(d, 4); kernels are
// compiled per class and a fit with d < D is computed with zero padding.
//
// Layout in HBM: the fits' rows are packed one fit after another (each fit
// starting on a 16-byte boundary); posteriors are component-major per fit
// (k x n); W_j = L_j^-1 is stored as a lower triangle whose rows are padded
// to multiples of 4 floats so the E-step reads it with 16-byte loads.
//
// Work items are built on the host when the batch is created (the shapes
// are fixed): E-step items of 128 P points, means items and covariance items
// of a per-class number of points (fem_em_batch_tuning; defaults kBMChunk,
// kBCChunk) x one range of <= 256 (component,
// TB x TB block) units.  Item lists are grouped by dimension class; each
// class is one launch per phase.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include <cuda.h>
#include <cuda_fp16.h>

#include "em_factor.cuh"
#include "fem_internal.cuh"
#include "tc_ptx.cuh"

namespace fem {
namespace {

constexpr int kBMaxD = 32;
constexpr int kBMaxK = 64;
constexpr int kBEThreads = 128;
constexpr int kBMThreads = 128;
constexpr int kBCThreads = 256;
constexpr int kBFThreads = 256;
constexpr int kBMChunk = 2048;   // points per means item
constexpr int kBCChunk = 4096;   // points per covariance item
constexpr int kBMTile = 128;     // points staged per means tile
constexpr int kBCTile = 16;      // points staged per covariance tile
constexpr int kBatchSyncEvery = 8;
constexpr int kTimeMarks = 15;   // timing events per sweep (see collect_timing)
constexpr int kClasses = 4;      // D = 4, 8, 16, 32

// padded lower triangle: row kk holds kk + 1 entries in 4 * ceil((kk + 1) / 4) floats
__host__ __device__ constexpr int tri_row(int kk) { return 4 * ((kk + 4) / 4); }
__host__ __device__ constexpr int tri_off(int kk) {
  int s = 0;
  for (int r = 0; r < kk; r++) s += tri_row(r);
  return s;
}
__host__ __device__ constexpr int class_tb(int D) { return D >= 16 ? 8 : 4; }
__host__ __device__ constexpr int class_nblk(int D) { return (D / class_tb(D)) * (D / class_tb(D) + 1) / 2; }
// covariance sums: D <= 16 by component owners (k_b_cov_own), D = 32 by TB x TB blocks (k_b_cov)
__host__ __device__ constexpr bool class_owner(int D) { return D <= 16; }
__host__ __device__ constexpr int own_S(int D) { return D >= 16 ? 2 : 1; }          // threads per component
__host__ __device__ constexpr int own_pairs(int D) { return D / 2 / own_S(D); }     // row pairs per thread
__host__ __device__ constexpr int own_NE(int D) { return own_pairs(D) * (D + 1); }  // sums per thread
__host__ __device__ constexpr int own_TP(int D) { return D >= 16 ? 32 : 128; }      // points per tile
int class_of(int d) { return d <= 4 ? 0 : d <= 8 ? 1 : d <= 16 ? 2 : 3; }
int class_dim(int c) { return 4 << c; }

// device descriptor of one fit
struct BFit {
  const float *X;        // n x d rows
  float *R;              // k x n, component-major
  int64_t n;
  int d, k, D;
  int nug;               // covariance unit ranges: ceil(k nblk / 256)
  int e_first, e_count;  // E-step items (global indices)
  int m_first, m_count;  // means items
  int64_t m_part;        // first means partial (doubles): m_count blocks of k (D + 4)
  int c_chunks;          // covariance chunks (items = c_chunks x nug)
  int64_t c_part;        // first covariance partial; chunk stride c_stride
  int64_t c_stride;
  double *pi, *mu, *sigma, *psum, *logc;   // k, k d, k d d, k, k
  float *muT, *WT, *logcT;                 // k D, k tri(D), k
  int64_t xrow;          // mixed form, d <= 32 class: first row in the FP16 split copies (-1: none)
  int wg;                // first 4-component W group of the tensor-core E-step
};

// per-fit training state
struct BState {
  int active;                 // still sweeping
  int status;                 // FEM_OK or the error that stopped the fit
  int iters;                  // EMAlgorithm's IterCounter
  int chol_failed;            // first failing component of this sweep (INT_MAX: none)
  unsigned long long cond;    // largest condition number of this sweep (bits of a double >= 0)
  double logl, prev;
  int fail_comp;
  int pad;
};

struct EItem { int fit, p0; };
struct MItem { int fit, p0, p1; int64_t part; };
struct CItem { int fit, p0, p1, u0, u1; int64_t part; };

__device__ __forceinline__ double bwarp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
// deterministic block sum, result in thread 0
template <int NT>
__device__ double bblock_sum(double v, double *red) {
  v = bwarp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; i++) s += red[i];
  return s;
}

__device__ __forceinline__ void blse_push(float l, float &mx, float &se) {
  if (l > mx) {
    se = se * expf(mx - l) + 1.f;
    mx = l;
  } else if (l > -INFINITY) {
    se += expf(l - mx);
  }
}

// 4-byte asynchronous global -> shared copy; `valid` false writes zero
__device__ __forceinline__ void cp_async4(float *dst, const float *src, bool valid) {
  const unsigned da = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(da), "l"(src), "r"(valid ? 4 : 0) : "memory");
}
// 16-byte asynchronous global -> shared copy (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async16(float *dst, const float *src) {
  const unsigned da = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(da), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// s_p += ||row KK of W . t_p||^2 for rows KK.. D-1 of a padded lower
// triangle W, P centred points; rows by compile-time recursion so every
// column bound is a constant, two interleaved accumulators per row for
// instruction-level parallelism
template <int D, int P, int KK>
__device__ __forceinline__ void tri_rows(const float (&t)[P][D], const float *__restrict__ w, float (&s)[P]) {
  float y0[P], y1[P];
#pragma unroll
  for (int p = 0; p < P; p++) y0[p] = 0.f, y1[p] = 0.f;
  const float *wr = w + tri_off(KK);
#pragma unroll
  for (int m4 = 0; m4 <= KK / 4; m4++) {
    const float4 wv = *reinterpret_cast<const float4 *>(wr + 4 * m4);
    const float we[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
    for (int e = 0; e < 4; e++) {
      if (4 * m4 + e <= KK) {
#pragma unroll
        for (int p = 0; p < P; p++) {
          if (m4 & 1) y1[p] = fmaf(t[p][4 * m4 + e], we[e], y1[p]);
          else y0[p] = fmaf(t[p][4 * m4 + e], we[e], y0[p]);
        }
      }
    }
  }
#pragma unroll
  for (int p = 0; p < P; p++) {
    const float y = y0[p] + y1[p];
    s[p] = fmaf(y, y, s[p]);
  }
  if constexpr (KK + 1 < D) tri_rows<D, P, KK + 1>(t, w, s);
}

// s_p = ||W t_p||^2
template <int D, int P>
__device__ __forceinline__ void tri_norms(const float (&t)[P][D], const float *__restrict__ w, float (&s)[P]) {
#pragma unroll
  for (int p = 0; p < P; p++) s[p] = 0.f;
  tri_rows<D, P, 0>(t, w, s);
}

// ================================================================ E-step
// MatrixEMBase::BlockDensities + PostProcessDensityMatrix
// (EM2/MatrixEM.cpp:39-51,69-81) for one item: 128 P points of one fit.
// The item's rows are staged once in shared memory, transposed (a column of
// 128 P values per dimension, stride kBEXs: conflict-free stores and reads).
// Components are staged kc at a time; per component each thread centres its
// P points on the mean, forms ||W_j (x - mu_j)||^2, writes l_ij to R and
// keeps an online log-sum-exp; a second pass turns l_ij into
// exp(l_ij - LSE_i).
constexpr int kBEP = 4;                          // points per thread
constexpr int kBEPoints = kBEThreads * kBEP;     // points per item
constexpr int kBEXs = kBEPoints + 1;             // transposed row stride (floats)

template <int D>
constexpr size_t estep_smem() {
  constexpr int KC = D >= 32 ? 8 : 16;
  return ((size_t)D * kBEXs + 2 * (size_t)((KC * tri_off(D) + KC * D + KC + 3) & ~3)) * sizeof(float);
}

template <int D, int P>
__global__ void __launch_bounds__(kBEThreads)
k_b_estep(const BFit *__restrict__ fits, const BState *__restrict__ state, const EItem *__restrict__ items,
          double *__restrict__ epart) {
  static_assert(P == kBEP, "points per thread");
  constexpr int TRI = tri_off(D);
  constexpr int KC = D >= 32 ? 8 : 16;
  constexpr int CB = KC * TRI + KC * D + KC;      // one component buffer: W, means, log coefficients
  constexpr int CBP = (CB + 3) & ~3;
  extern __shared__ __align__(16) float sXt[];   // D x kBEXs, then two component buffers
  __shared__ double red[kBEThreads / 32];
  const EItem item = items[blockIdx.x];
  if (!state[item.fit].active) return;
  const BFit &F = fits[item.fit];
  const float *__restrict__ X = F.X;
  float *__restrict__ R = F.R;
  const int64_t n = F.n;
  const int d = F.d, K = F.k, tid = threadIdx.x;
  float *cbuf = sXt + D * kBEXs;
  // components [j0, j0 + kc) into buffer b (16-byte copies; W rows and means are 16-byte multiples)
  auto stage = [&](int b, int j0) {
    const int kc = min(KC, K - j0);
    float *w = cbuf + b * CBP, *m = w + KC * TRI, *l = m + KC * D;
    for (int e = tid; e < kc * TRI / 4; e += kBEThreads) cp_async16(w + 4 * e, F.WT + (size_t)j0 * TRI + 4 * e);
    for (int e = tid; e < kc * D / 4; e += kBEThreads) cp_async16(m + 4 * e, F.muT + (size_t)j0 * D + 4 * e);
    for (int e = tid; e < kc; e += kBEThreads) cp_async4(l + e, F.logcT + j0 + e, true);
    cp_async_commit();
  };
  stage(0, 0);
  const int npts = (int)min((int64_t)kBEPoints, n - item.p0);
  // rows -> transposed columns (zero past the last point and past column d)
  if (d == D) {
    const float4 *src = reinterpret_cast<const float4 *>(X + (size_t)item.p0 * D);
    for (int e = tid; e < kBEPoints * D / 4; e += kBEThreads) {
      const int pt = (4 * e) / D, q = (4 * e) % D;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (pt < npts) v = src[e];
      sXt[(q + 0) * kBEXs + pt] = v.x;
      sXt[(q + 1) * kBEXs + pt] = v.y;
      sXt[(q + 2) * kBEXs + pt] = v.z;
      sXt[(q + 3) * kBEXs + pt] = v.w;
    }
  } else {
    const float *src = X + (size_t)item.p0 * d;
    for (int e = tid; e < kBEPoints * D; e += kBEThreads) {
      const int pt = e / D, q = e - pt * D;
      sXt[q * kBEXs + pt] = (pt < npts && q < d) ? src[(size_t)pt * d + q] : 0.f;
    }
  }
  int64_t idx[P];
  bool valid[P];
#pragma unroll
  for (int p = 0; p < P; p++) {
    idx[p] = (int64_t)item.p0 + tid + p * kBEThreads;
    valid[p] = idx[p] < n;
  }
  float mx[P], se[P];
#pragma unroll
  for (int p = 0; p < P; p++) mx[p] = -INFINITY, se[p] = 0.f;
  int b = 0;
  for (int j0 = 0; j0 < K; j0 += KC, b ^= 1) {
    const int kc = min(KC, K - j0);
    if (j0 + KC < K) stage(b ^ 1, j0 + KC);
    else cp_async_commit();
    cp_async_wait_prev();
    __syncthreads();
    const float *sW = cbuf + b * CBP, *smu = sW + KC * TRI, *slc = smu + KC * D;
    for (int jj = 0; jj < kc; jj++) {
      const float *m = smu + jj * D;
      float t[P][D];
#pragma unroll
      for (int q = 0; q < D; q++) {
        const float mq = m[q];
#pragma unroll
        for (int p = 0; p < P; p++) t[p][q] = sXt[q * kBEXs + tid + p * kBEThreads] - mq;
      }
      float s[P];
      tri_norms<D, P>(t, sW + jj * TRI, s);
      const float lc = slc[jj];
      float *Rj = R + (size_t)(j0 + jj) * n;
#pragma unroll
      for (int p = 0; p < P; p++) {
        const float l = lc - 0.5f * s[p];
        if (valid[p]) Rj[idx[p]] = l;
        blse_push(l, mx[p], se[p]);
      }
    }
    __syncthreads();
  }
  cp_async_wait_all();
  double v = 0.0;
  float lse[P];
#pragma unroll
  for (int p = 0; p < P; p++) {
    lse[p] = mx[p] + logf(se[p]);
    if (valid[p]) v += (double)lse[p];
  }
#pragma unroll 4
  for (int j = 0; j < K; j++) {
    float *Rj = R + (size_t)j * n;
#pragma unroll
    for (int p = 0; p < P; p++)
      if (valid[p]) Rj[idx[p]] = expf(Rj[idx[p]] - lse[p]);
  }
  const double sum = bblock_sum<kBEThreads>(v, red);
  if (tid == 0) epart[blockIdx.x] = sum;
}

// ======================================================= M-step: means
// SimpleMatrixEM::doMStep means part (EM2/MatrixEM.cpp:319-343) for one item:
// sums_j[c] = sum_i r_ij [x_i | 1][c] over the item's points, as a K x (D+4)
// block of FP64 partials (column D holds PosteriorSum_j).  Threads own 4 x 4
// micro-tiles of (component, column); when there are fewer micro-tiles than
// threads, point groups split each tile's points and are summed at the end.
// Tiles of kBMTile points are copied with cp.async one tile ahead into two
// shared buffers (rows x (D + 4) with the ones column, posteriors point-major
// with an odd stride).  FP32 sums over the item.
template <int D>
__host__ __device__ constexpr size_t means_buf_floats(int kmax) {
  return (((size_t)kBMTile * (D + 4) + (size_t)kBMTile * (((kmax + 3) & ~3) + 1)) + 3) & ~(size_t)3;
}

template <int D>
__global__ void __launch_bounds__(kBMThreads)
k_b_means(const BFit *__restrict__ fits, const BState *__restrict__ state, const MItem *__restrict__ items,
          double *__restrict__ mpart, int kmax) {
  constexpr int XC = D + 4, NQB = XC / 4, TP = kBMTile;
  constexpr int UPT = (kBMaxK / 4 * NQB + kBMThreads - 1) / kBMThreads;
  extern __shared__ __align__(16) float msm[];
  const MItem item = items[blockIdx.x];
  if (!state[item.fit].active) return;
  const BFit &F = fits[item.fit];
  const float *__restrict__ X = F.X;
  const float *__restrict__ R = F.R;
  const int64_t n = F.n;
  const int d = F.d, K = F.k, tid = threadIdx.x;
  const int K4 = (K + 3) & ~3, SR = ((kmax + 3) & ~3) + 1, nmt = (K4 / 4) * NQB;
  const size_t bufsz = means_buf_floats<D>(kmax);
  const bool grouped = nmt <= kBMThreads;
  const int UG = grouped ? (nmt + 31) & ~31 : kBMThreads;
  const int MG = grouped ? kBMThreads / UG : 1;
  const int g = grouped ? tid / UG : 0;
  const bool gok = g < MG;
  int mt[UPT];
#pragma unroll
  for (int u = 0; u < UPT; u++) mt[u] = grouped ? (u == 0 ? tid % UG : nmt) : tid + u * kBMThreads;
  // columns d..D-1 and D+1..D+3 stay zero; posterior columns K..K4-1 too
  for (size_t e = tid; e < 2 * bufsz; e += kBMThreads) msm[e] = 0.f;
  __syncthreads();
  auto stage = [&](int buf, int t0) {
    float *sx = msm + buf * bufsz, *sr = sx + TP * XC;
    const int tp = min(TP, item.p1 - t0);
    for (int e = tid; e < TP * d; e += kBMThreads) {
      const int p = e / d, c = e - p * d;
      cp_async4(sx + p * XC + c, X + (p < tp ? (size_t)(t0 + p) * d + c : 0), p < tp);
    }
    for (int e = tid; e < K * TP; e += kBMThreads) {
      const int j = e / TP, p = e - j * TP;
      cp_async4(sr + p * SR + j, R + (size_t)j * n + (p < tp ? t0 + p : 0), p < tp);
    }
    for (int p = tid; p < TP; p += kBMThreads) sx[p * XC + D] = p < tp ? 1.f : 0.f;
    cp_async_commit();
  };
  float acc[UPT][4][4];
#pragma unroll
  for (int u = 0; u < UPT; u++)
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) acc[u][a][b] = 0.f;
  stage(0, item.p0);
  int buf = 0;
  for (int t0 = item.p0; t0 < item.p1; t0 += TP, buf ^= 1) {
    if (t0 + TP < item.p1) stage(buf ^ 1, t0 + TP);
    else cp_async_commit();
    cp_async_wait_prev();
    __syncthreads();
    const float *sx = msm + buf * bufsz, *sr = sx + TP * XC;
    if (gok) {
#pragma unroll
      for (int u = 0; u < UPT; u++) {
        if (mt[u] < nmt) {
          const int jb = mt[u] / NQB, qb = mt[u] - jb * NQB;
          for (int p = g; p < TP; p += MG) {
            const float *rp = sr + p * SR + 4 * jb;
            const float4 xv = *reinterpret_cast<const float4 *>(sx + p * XC + 4 * qb);
            const float xs[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
            for (int a = 0; a < 4; a++) {
              const float r = rp[a];
#pragma unroll
              for (int b = 0; b < 4; b++) acc[u][a][b] = fmaf(r, xs[b], acc[u][a][b]);
            }
          }
        }
      }
    }
    __syncthreads();
  }
  if (MG > 1) {
    // point groups 1.. hand their sums to group 0 (in group order)
    float *red = msm;
    if (gok && g > 0 && mt[0] < nmt)
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) red[((g - 1) * UG + mt[0]) * 16 + a * 4 + b] = acc[0][a][b];
    __syncthreads();
    if (g == 0 && mt[0] < nmt)
      for (int gg = 1; gg < MG; gg++)
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int b = 0; b < 4; b++) acc[0][a][b] += red[((gg - 1) * UG + mt[0]) * 16 + a * 4 + b];
  }
  if (g != 0) return;
  double *o = mpart + item.part;
#pragma unroll
  for (int u = 0; u < UPT; u++) {
    if (mt[u] < nmt) {
      const int jb = mt[u] / NQB, qb = mt[u] - jb * NQB;
#pragma unroll
      for (int a = 0; a < 4; a++) {
        const int j = 4 * jb + a;
        if (j < K)
#pragma unroll
          for (int b = 0; b < 4; b++) o[(size_t)j * XC + 4 * qb + b] = (double)acc[u][a][b];
      }
    }
  }
}

// PosteriorSum, Means = MeanSums / PosteriorSum, Probs = PosteriorSum / N
// (EM2/MatrixEM.cpp:341-343,375) and LogL = sum_i LSE_i, one CTA per fit;
// partials summed in item order.
template <int NT>
__global__ void __launch_bounds__(NT)
k_b_final_means(const BFit *__restrict__ fits, BState *__restrict__ state, const double *__restrict__ epart,
                const double *__restrict__ mpart) {
  __shared__ double red[NT / 32];
  const int f = blockIdx.x, tid = threadIdx.x;
  if (!state[f].active) return;
  const BFit &F = fits[f];
  const int K = F.k, d = F.d, D = F.D, XC = D + 4;
  double v = 0.0;
  for (int e = tid; e < F.e_count; e += NT) v += epart[F.e_first + e];
  const double ll = bblock_sum<NT>(v, red);
  if (tid == 0) state[f].logl = ll;
  const double *mp = mpart + F.m_part;
  const size_t stride = (size_t)K * XC;
  for (int j = tid; j < K; j += NT) {
    double s = 0.0;
    for (int c = 0; c < F.m_count; c++) s += mp[c * stride + (size_t)j * XC + D];
    F.psum[j] = s;
    F.pi[j] = s / (double)F.n;
  }
  __syncthreads();
  for (int e = tid; e < K * D; e += NT) {
    const int j = e / D, q = e - j * D;
    if (q < d) {
      double s = 0.0;
      for (int c = 0; c < F.m_count; c++) s += mp[c * stride + (size_t)j * XC + q];
      const double m = s / F.psum[j];
      F.mu[(size_t)j * d + q] = m;
      F.muT[e] = (float)m;
    } else {
      F.muT[e] = 0.f;
    }
  }
}

// ================================================== M-step: covariances
// MatrixEMBase::ComputeWeightedTempDataset + BlockCovariances
// (EM2/MatrixEM.cpp:53-67,90-99) for one item: z = sqrt(r_ij) (x_i - mu_j)
// around the new means, CovSum_j += z z^T over the upper block triangle.
// A unit is one TB x TB block of one component; the item's units
// [u0, u1) take UG = roundup32(u1 - u0) threads and the CTA's 256 / UG
// point groups split each tile's points.  Per tile of kBCTile points the x
// rows and sqrt(r) are staged in shared memory (loaded into registers one
// tile ahead, so the loads overlap the previous tile's work), z is built
// there for the item's components, then each unit accumulates its block.
// FP32 sums over the item's points; each (group, unit) writes its TB x TB
// block as FP64 partials.
template <int D>
struct CovGeom {
  static constexpr int TB = class_tb(D), NB = D / TB, NBLK = class_nblk(D);
  static constexpr int ZP = D + 4;                                   // z / x row pitch (floats)
  static constexpr int CJMAX = kBMaxK < 256 / NBLK + 2 ? kBMaxK : 256 / NBLK + 2;
  static constexpr int ZCS = kBCTile * ZP + 4;                       // z stride per component (bank skew)
  static constexpr int XT = kBCTile * D;                             // x tile values
  static constexpr int XPT = (XT + kBCThreads - 1) / kBCThreads;
  static constexpr int RPT = (CJMAX * kBCTile + kBCThreads - 1) / kBCThreads;
  // smem floats: mu (CJ x ZP), x tile (TP x ZP), w (CJ x TP), z (CJ x ZCS)
  static constexpr size_t floats(int cj) {
    return (size_t)cj * ZP + (size_t)kBCTile * ZP + (((size_t)cj * kBCTile + 3) & ~(size_t)3) + (size_t)cj * ZCS;
  }
};

template <int D>
__global__ void __launch_bounds__(kBCThreads, 2)
k_b_cov(const BFit *__restrict__ fits, const BState *__restrict__ state, const CItem *__restrict__ items,
        double *__restrict__ cpart) {
  using G = CovGeom<D>;
  constexpr int TB = G::TB, NB = G::NB, NBLK = G::NBLK, ZP = G::ZP, ZCS = G::ZCS, TP = kBCTile;
  extern __shared__ __align__(16) float csm[];
  const CItem item = items[blockIdx.x];
  if (!state[item.fit].active) return;
  const BFit &F = fits[item.fit];
  const float *__restrict__ X = F.X;
  const float *__restrict__ R = F.R;
  const int64_t n = F.n;
  const int d = F.d, tid = threadIdx.x;
  const int nunits = item.u1 - item.u0;
  const int UG = (nunits + 31) & ~31, NG = kBCThreads / UG;
  const int ul = tid % UG, g = tid / UG;
  const bool act = ul < nunits && g < NG;
  const int j_lo = item.u0 / NBLK, j_hi = (item.u1 - 1) / NBLK, CJ = j_hi - j_lo + 1;
  float *smu = csm;                                   // CJ x ZP
  float *sx = smu + (size_t)CJ * ZP;                  // TP x ZP
  float *sw = sx + (size_t)TP * ZP;                   // CJ x TP
  float *sZ = sw + (((size_t)CJ * TP + 3) & ~(size_t)3);   // CJ x ZCS
  int cj = 0, bi = 0, bj = 0;
  if (act) {
    const int unit = item.u0 + ul;
    const int j = unit / NBLK;
    int b = unit - j * NBLK;
    while (b >= NB - bi) {
      b -= NB - bi;
      bi++;
    }
    bj = bi + b;
    cj = j - j_lo;
  }
  for (int e = tid; e < CJ * ZP; e += kBCThreads) {
    const int jj = e / ZP, q = e - jj * ZP;
    smu[e] = q < D ? F.muT[(size_t)(j_lo + jj) * D + q] : 0.f;
  }
  // register prefetch of one tile's x values and posteriors
  float xr[G::XPT], rr[G::RPT];
  auto fetch = [&](int t0) {
    const int tp = min(TP, item.p1 - t0);
#pragma unroll
    for (int u = 0; u < G::XPT; u++) {
      const int e = tid + u * kBCThreads, p = e / D, q = e - p * D;
      xr[u] = (e < G::XT && p < tp && q < d) ? X[(size_t)(t0 + p) * d + q] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < G::RPT; u++) {
      const int e = tid + u * kBCThreads, jj = e / TP, p = e - jj * TP;
      rr[u] = (jj < CJ && p < tp) ? R[(size_t)(j_lo + jj) * n + t0 + p] : 0.f;
    }
  };
  fetch(item.p0);
  float acc[TB][TB];
#pragma unroll
  for (int a = 0; a < TB; a++)
#pragma unroll
    for (int b = 0; b < TB; b++) acc[a][b] = 0.f;
  for (int t0 = item.p0; t0 < item.p1; t0 += TP) {
    __syncthreads();
#pragma unroll
    for (int u = 0; u < G::XPT; u++) {
      const int e = tid + u * kBCThreads, p = e / D, q = e - p * D;
      if (e < G::XT) sx[p * ZP + q] = xr[u];
    }
#pragma unroll
    for (int u = 0; u < G::RPT; u++) {
      const int e = tid + u * kBCThreads;
      if (e < CJ * TP) sw[e] = sqrtf(rr[u]);
    }
    __syncthreads();
    if (t0 + TP < item.p1) fetch(t0 + TP);
#pragma unroll 1
    for (int e = tid; e < CJ * TP * (D / 4); e += kBCThreads) {
      const int row = e / (D / 4), q4 = e - row * (D / 4);
      const int jj = row / TP, p = row - jj * TP;
      const float w = sw[row];
      const float4 xv = *reinterpret_cast<const float4 *>(sx + p * ZP + 4 * q4);
      const float4 mv = *reinterpret_cast<const float4 *>(smu + jj * ZP + 4 * q4);
      float4 z;
      z.x = w * (xv.x - mv.x);
      z.y = w * (xv.y - mv.y);
      z.z = w * (xv.z - mv.z);
      z.w = w * (xv.w - mv.w);
      *reinterpret_cast<float4 *>(sZ + (size_t)jj * ZCS + p * ZP + 4 * q4) = z;
    }
    __syncthreads();
    if (act) {
      const float *zb = sZ + (size_t)cj * ZCS;
#pragma unroll 1
      for (int p = g; p < TP; p += NG) {
        const float *zr = zb + p * ZP;
        float va[TB], vb[TB];
#pragma unroll
        for (int a4 = 0; a4 < TB / 4; a4++) {
          const float4 u = *reinterpret_cast<const float4 *>(zr + bi * TB + 4 * a4);
          const float4 v = *reinterpret_cast<const float4 *>(zr + bj * TB + 4 * a4);
          va[4 * a4 + 0] = u.x, va[4 * a4 + 1] = u.y, va[4 * a4 + 2] = u.z, va[4 * a4 + 3] = u.w;
          vb[4 * a4 + 0] = v.x, vb[4 * a4 + 1] = v.y, vb[4 * a4 + 2] = v.z, vb[4 * a4 + 3] = v.w;
        }
#pragma unroll
        for (int a = 0; a < TB; a++)
#pragma unroll
          for (int b = 0; b < TB; b++) acc[a][b] = fmaf(va[a], vb[b], acc[a][b]);
      }
    }
  }
  if (act) {
    double *o = cpart + item.part + ((size_t)g * nunits + ul) * (TB * TB);
#pragma unroll
    for (int a = 0; a < TB; a++)
#pragma unroll
      for (int b = 0; b < TB; b++) o[a * TB + b] = (double)acc[a][b];
  }
}

// Partial geometry of covariance unit range `ug` of a fit with k components
// in class D: units [u0, u1), ng point groups, per doubles per unit; the
// range's partials are ng x (u1 - u0) x per doubles.  Block layout (D = 32):
// a unit is one TB x TB block of one component, ranges of <= 256 units.
// Owner layout (D <= 16): one range whose units are the k components, each
// owned by own_S(D) threads of own_NE(D) sums.
__host__ __device__ inline void unit_range(int k, int D, int ug, int *u0, int *u1, int *ng, int *per) {
  if (class_owner(D)) {
    *u0 = 0;
    *u1 = k;
    *ng = 256 / (own_S(D) * ((k + 31) & ~31));
    *per = own_S(D) * own_NE(D);
    return;
  }
  const int total = k * class_nblk(D);
  *u0 = ug * 256;
  *u1 = min(total, *u0 + 256);
  const int UG = (*u1 - *u0 + 31) & ~31;
  *ng = 256 / UG;
  *per = class_tb(D) * class_tb(D);
}

// one point's contribution r u u^T to the sums of row pairs I.. of the
// thread set SS: pair q covers rows q (columns q..D-1) and D-1-q (columns
// D-1-q..D-1), D + 1 sums; compile-time recursion keeps every index constant
template <int D, int SS, int I>
__device__ __forceinline__ void own_pairs_acc(const float (&u)[D], float r, float (&acc)[own_NE(D)]) {
  constexpr int S = own_S(D), q = SS + S * I, q2 = D - 1 - q, base = I * (D + 1);
  const float ra = r * u[q], rb = r * u[q2];
#pragma unroll
  for (int c = q; c < D; c++) acc[base + c - q] = fmaf(ra, u[c], acc[base + c - q]);
#pragma unroll
  for (int c = q2; c < D; c++) acc[base + (D - q) + c - q2] = fmaf(rb, u[c], acc[base + (D - q) + c - q2]);
  if constexpr (I + 1 < own_pairs(D)) own_pairs_acc<D, SS, I + 1>(u, r, acc);
}

// shared memory of k_b_cov_own<D> for classes with at most kmax components:
// two buffers of (TP x D rows, kmax x (TP + 1) posteriors); the odd row
// stride keeps the lanes of a warp (consecutive components, one point) in
// different banks
__host__ __device__ constexpr size_t own_buf_floats(int D, int kmax) {
  return ((size_t)own_TP(D) * D + (size_t)kmax * (own_TP(D) + 1) + 3) & ~(size_t)3;
}

// MatrixEMBase::ComputeWeightedTempDataset + BlockCovariances
// (EM2/MatrixEM.cpp:53-67,90-99) for D <= 16: CovSum_j += r_ij u u^T with
// u = x_i - mu_j formed on the fly from a staged tile of rows.  A component
// is owned by own_S(D) threads (a warp-uniform split of its row pairs), the
// CTA's 256 / (own_S roundup32(k)) point groups split each tile's points.
// Tiles are copied asynchronously one tile ahead into two shared buffers.
// FP32 sums over the item; partials [group][thread set][component][own_NE]
// in FP64.
template <int D>
__global__ void __launch_bounds__(kBCThreads, D >= 16 ? 1 : 2)
k_b_cov_own(const BFit *__restrict__ fits, const BState *__restrict__ state, const CItem *__restrict__ items,
            double *__restrict__ cpart, int kmax) {
  constexpr int S = own_S(D), NE = own_NE(D), TP = own_TP(D);
  extern __shared__ __align__(16) float osm[];
  const CItem item = items[blockIdx.x];
  if (!state[item.fit].active) return;
  const BFit &F = fits[item.fit];
  const float *__restrict__ X = F.X;
  const float *__restrict__ R = F.R;
  const int64_t n = F.n;
  const int d = F.d, K = F.k, tid = threadIdx.x;
  const int KG = (K + 31) & ~31, UG = S * KG, NG = kBCThreads / UG;
  const int ul = tid % UG, g = tid / UG, ts = ul / KG, j = ul - ts * KG;
  const bool act = j < K && g < NG;
  const size_t bufsz = own_buf_floats(D, kmax);
  float mu[D];
#pragma unroll
  for (int q = 0; q < D; q++) mu[q] = act ? F.muT[(size_t)j * D + q] : 0.f;
  float acc[NE];
#pragma unroll
  for (int e = 0; e < NE; e++) acc[e] = 0.f;
  // one tile of rows (TP x D, zero past d and past the item) and posteriors (K x TP)
  auto stage = [&](int buf, int t0) {
    float *sx = osm + buf * bufsz, *sr = sx + TP * D;
    const int tp = min(TP, item.p1 - t0);
    for (int e = tid; e < TP * D; e += kBCThreads) {
      const int p = e / D, q = e - p * D;
      const bool v = p < tp && q < d;
      cp_async4(sx + e, X + (v ? (size_t)(t0 + p) * d + q : 0), v);
    }
    for (int e = tid; e < K * TP; e += kBCThreads) {
      const int jj = e / TP, p = e - jj * TP;
      const bool v = p < tp;
      cp_async4(sr + jj * (TP + 1) + p, R + (size_t)jj * n + (v ? t0 + p : 0), v);
    }
    cp_async_commit();
  };
  stage(0, item.p0);
  int buf = 0;
  for (int t0 = item.p0; t0 < item.p1; t0 += TP, buf ^= 1) {
    if (t0 + TP < item.p1) stage(buf ^ 1, t0 + TP);
    else cp_async_commit();                 // an empty group keeps the wait count uniform
    cp_async_wait_prev();
    __syncthreads();
    const float *sx = osm + buf * bufsz, *sr = sx + TP * D;
    const int tp = min(TP, item.p1 - t0);
    if (act) {
      for (int p = g; p < tp; p += NG) {
        const float r = sr[j * (TP + 1) + p];
        float u[D];
#pragma unroll
        for (int q4 = 0; q4 < D / 4; q4++) {
          const float4 xv = *reinterpret_cast<const float4 *>(sx + p * D + 4 * q4);
          u[4 * q4 + 0] = xv.x - mu[4 * q4 + 0];
          u[4 * q4 + 1] = xv.y - mu[4 * q4 + 1];
          u[4 * q4 + 2] = xv.z - mu[4 * q4 + 2];
          u[4 * q4 + 3] = xv.w - mu[4 * q4 + 3];
        }
        if constexpr (S == 1) {
          own_pairs_acc<D, 0, 0>(u, r, acc);
        } else {
          if (ts == 0) own_pairs_acc<D, 0, 0>(u, r, acc);
          else own_pairs_acc<D, 1, 0>(u, r, acc);
        }
      }
    }
    __syncthreads();
  }
  if (act) {
    double *o = cpart + item.part + ((size_t)(g * S + ts) * K + j) * NE;
#pragma unroll
    for (int e = 0; e < NE; e++) o[e] = (double)acc[e];
  }
}

// ======================================================= factorisation
// Covs_j = CovSum_j / PosteriorSum_j (EM2/MatrixEM.cpp:370-373) from the
// covariance partials (when `reduce`), then RegularizeCovariances +
// NormalDensity::Init + CalcLogCoeffs (EM2/EMAlgorithm.cpp:237-244,
// EM2/NormalDensity.cpp:43-65, EM2/MatrixEM.cpp:83-87) in FP64, and with
// `svd` the condition number (EM2/NormalDensity.cpp:67-71).  One CTA per
// (fit, component); the factor lives in shared memory.
__global__ void __launch_bounds__(kBFThreads)
k_b_factor(const BFit *__restrict__ fits, BState *__restrict__ state, const int2 *__restrict__ comps,
           const double *__restrict__ cpart, double reg, int reduce, int svd) {
  __shared__ double sA[kBMaxD * kBMaxD];
  __shared__ double sWi[kBMaxD * kBMaxD];
  const int2 fc = comps[blockIdx.x];
  const int f = fc.x, j = fc.y, tid = threadIdx.x;
  if (!state[f].active) return;
  const BFit &F = fits[f];
  const int d = F.d, D = F.D, K = F.k;
  double *S = F.sigma + (size_t)j * d * d;
  if (reduce) {
    const double inv = 1.0 / F.psum[j];
    if (class_owner(D)) {
      const int Sd = own_S(D), NE = own_NE(D);
      int u0 = 0, u1 = 0, ng = 0, per = 0;
      unit_range(K, D, 0, &u0, &u1, &ng, &per);
      for (int e = tid; e < d * d; e += kBFThreads) {
        const int a = e / d, c = e - a * d;
        if (a > c) continue;
        const bool first = a < D / 2;
        const int q = first ? a : D - 1 - a;
        const int ts = q % Sd, i = q / Sd;
        const int w = i * (D + 1) + (first ? c - a : (D - q) + (c - a));
        double s2 = 0.0;
        for (int ch = 0; ch < F.c_chunks; ch++) {
          const double *pp = cpart + F.c_part + ch * F.c_stride + ((size_t)ts * K + j) * NE + w;
          for (int gg = 0; gg < ng; gg++) s2 += pp[(size_t)gg * Sd * K * NE];
        }
        s2 *= inv;
        S[(size_t)a * d + c] = s2;
        S[(size_t)c * d + a] = s2;
      }
    } else {
      const int TB = class_tb(D), NB = D / TB, NBLK = class_nblk(D), per = TB * TB;
      for (int e = tid; e < NBLK * per; e += kBFThreads) {
        const int b = e / per, w = e - b * per;
        int bi = 0, bb = b;
        while (bb >= NB - bi) {
          bb -= NB - bi;
          bi++;
        }
        const int bj = bi + bb;
        const int a = bi * TB + w / TB, c = bj * TB + (w % TB);
        if (a > c || c >= d) continue;
        const int unit = j * NBLK + b, ug = unit / 256, ul = unit - ug * 256;
        int64_t off = 0;
        int u0 = 0, u1 = 0, ng = 0, pr = 0;
        for (int q = 0; q < ug; q++) {
          unit_range(K, D, q, &u0, &u1, &ng, &pr);
          off += (int64_t)ng * (u1 - u0) * pr;
        }
        unit_range(K, D, ug, &u0, &u1, &ng, &pr);
        const int nu = u1 - u0;
        double s2 = 0.0;
        for (int ch = 0; ch < F.c_chunks; ch++) {
          const double *pp = cpart + F.c_part + ch * F.c_stride + off + (size_t)ul * per + w;
          for (int gg = 0; gg < ng; gg++) s2 += pp[(size_t)gg * nu * per];
        }
        s2 *= inv;
        S[(size_t)a * d + c] = s2;
        S[(size_t)c * d + a] = s2;
      }
    }
    __syncthreads();
  }
  if (reg != 0.0) block_regularize(S, d, reg);
  if (!block_cholesky(S, d, sA)) {
    if (tid == 0) atomicMin(&state[f].chol_failed, j);
    return;
  }
  block_lower_inverse(sA, d, sWi);
  const double ld = block_chol_logdet(sA, d);
  if (tid == 0) {
    const double lc = log(F.pi[j]) - 0.5 * (double)d * log(2.0 * M_PI) - 0.5 * ld;
    F.logc[j] = lc;
    F.logcT[j] = (float)lc;
  }
  const int TRI = tri_off(D);
  float *Wt = F.WT + (size_t)j * TRI;
  for (int e = tid; e < TRI; e += kBFThreads) {
    int kk = 0, off = 0;
    while (off + tri_row(kk) <= e) off += tri_row(kk++);
    const int m = e - off;
    Wt[e] = (kk < d && m <= kk) ? (float)sWi[kk * d + m] : 0.f;
  }
  if (svd) {
    __syncthreads();
    for (int e = tid; e < d * d; e += kBFThreads) {
      const int r = e / d, c = e - r * d;
      sA[e] = (c <= r) ? S[e] : S[(size_t)c * d + r];
    }
    __syncthreads();
    const double cond = block_jacobi_cond(sA, d);
    if (tid == 0) atomicMax(&state[f].cond, (unsigned long long)__double_as_longlong(cond));
  }
}

// the end of one sweep of TrainNoCopy's loop (EM2/EMAlgorithm.cpp:167-185)
// for every active fit: a failed factorisation or a condition number above
// AbortThr stops the fit with IterCounter = it; otherwise LogL and e go to
// the traces and |dL/L| < Eps or MaxSweeps stops it with it + 1.  it = 0 is
// the factorisation before the first sweep.  One CTA; *nactive counts the
// fits still sweeping.
__global__ void __launch_bounds__(1024)
k_b_sweep_end(BState *__restrict__ state, int nfits, int it, int max_sweeps, double eps, double abort_thr,
              int svd, double *__restrict__ trace, double *__restrict__ etrace, int cap, int *nactive) {
  __shared__ double red[32];
  double cnt = 0.0;
  for (int f = threadIdx.x; f < nfits; f += 1024) {
    BState &s = state[f];
    if (!s.active) continue;
    if (s.chol_failed != INT_MAX) {
      s.status = FEM_ERR_CHOLESKY;
      s.fail_comp = s.chol_failed;
      s.iters = it;
      s.active = 0;
      continue;
    }
    if (svd) {
      const double cond = __longlong_as_double((long long)s.cond);
      s.cond = 0ull;
      if (cond > abort_thr) {
        s.status = FEM_ERR_COND_ABORT;
        s.iters = it;
        s.active = 0;
        continue;
      }
    }
    if (it > 0) {
      const double logl = s.logl;
      double e = fabs((logl - s.prev) / logl);
      if (logl < s.prev) e = 0.0;
      if (it - 1 < cap) {
        trace[(size_t)f * cap + it - 1] = logl;
        etrace[(size_t)f * cap + it - 1] = e;
      }
      s.prev = logl;
      s.iters = it + 1;
      if (e < eps || it >= max_sweeps) {
        s.active = 0;
        continue;
      }
    }
    cnt += 1.0;
  }
  const double total = bblock_sum<1024>(cnt, red);
  if (threadIdx.x == 0) *nactive = (int)total;
}


// ================================================ mixed form: tensor-core E-step
// For the d <= 32 class of a batch created with FEM_PREC_MIXED, the E-step of
// each 512-point item runs on the tensor cores: four 128-point tiles, each
// against the fit's components in groups of 4 (128 accumulator columns), in
// FP16 x 3 split products (x_h W_l, x_l W_h, x_h W_h) with FP32 accumulation,
// as the single-fit E-step (em_tc.cu) does at d <= 64.  Rows are zero-padded
// to 64 FP16 columns (128-byte swizzled operand rows); a group's 128 W rows are
// ordered [outputs 16..31 of its 4 components | outputs 0..15], so the second
// 16-wide k-step (inputs 16..31, lower triangle) needs only the first 64.
// The epilogue writes the same FP32 posteriors and per-item LogL partials as
// k_b_estep, so the rest of the sweep is unchanged.
constexpr int kTT = 128;            // points per tile
constexpr int kTWS = 4;             // W group ring
constexpr int kTThreads = 192;      // warp 0 TMA, 1 MMA, 2..5 epilogue
constexpr int kTClass = 3;          // the d <= 32 class
struct __align__(1024) BTSmem {
  __half xh[2][kTT * 64], xl[2][kTT * 64];
  __half wh[kTWS][128 * 64], wl[kTWS][128 * 64];
  uint64_t x_full[2], x_empty[2], w_full[kTWS], w_empty[kTWS], acc_full[2], acc_empty[2], mma_done;
  uint32_t tmem_base;
  double red[2][4];
};
static_assert(sizeof(BTSmem) + 1024 <= 232448, "batched tensor-core E-step shared memory");

// x -> FP16 hi / lo, rows padded to 64 columns; blockIdx.y = the class's fit
__global__ void k_bt_split(const BFit *__restrict__ fits, const int *__restrict__ tfits, __half *__restrict__ Xh,
                           __half *__restrict__ Xl) {
  const BFit &F = fits[tfits[blockIdx.y]];
  const int64_t tot = F.n * 64;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e >> 6;
    const int c = (int)(e & 63);
    const float x = c < F.d ? F.X[i * F.d + c] : 0.f;
    const __half h = __float2half_rn(x);
    Xh[(F.xrow + i) * 64 + c] = h;
    Xl[(F.xrow + i) * 64 + c] = __float2half_rn(x - __half2float(h));
  }
}

// per 4-component group: W = L^-1 (from the FP32 factor) as FP16 hi / lo in
// the tile order above, b = W mu (FP64 sum), log coefficients as float hi + lo
// (-inf for padding components)
__global__ void __launch_bounds__(128)
k_bt_prep(const BFit *__restrict__ fits, const int2 *__restrict__ tgroups, __half *__restrict__ Wh,
          __half *__restrict__ Wl, float *__restrict__ bias, float *__restrict__ chi, float *__restrict__ clo) {
  const int2 fg = tgroups[blockIdx.x];
  const BFit &F = fits[fg.x];
  const int r = threadIdx.x, grp = F.wg + fg.y;
  const int h = r >> 6, q = (r & 63) >> 4, t = r & 15;
  const int k = h == 0 ? 16 + t : t, j = 4 * fg.y + q;
  const bool live = j < F.k && k < F.d;
  constexpr int TRI = tri_off(32);
  const float *w = F.WT + (size_t)j * TRI + tri_off(k);
  double bsum = 0.0;
  for (int e = 0; e < 64; e++) {
    const float v = (live && e <= k && e < F.d) ? w[e] : 0.f;
    const __half vh = __float2half_rn(v);
    Wh[((size_t)grp * 128 + r) * 64 + e] = vh;
    Wl[((size_t)grp * 128 + r) * 64 + e] = __float2half_rn(v - __half2float(vh));
    if (live && e <= k && e < F.d) bsum += (double)v * F.mu[(size_t)j * F.d + e];
  }
  bias[(size_t)grp * 128 + r] = (float)bsum;
  if (r < 4) {
    const int jj = 4 * fg.y + r;
    const double lc = jj < F.k ? F.logc[jj] : 0.0;
    chi[(size_t)grp * 4 + r] = jj < F.k ? (float)lc : -INFINITY;
    clo[(size_t)grp * 4 + r] = jj < F.k ? (float)(lc - (double)(float)lc) : 0.f;
  }
}

__global__ void __launch_bounds__(kTThreads, 1)
k_bt_estep(const __grid_constant__ CUtensorMap tm_xh, const __grid_constant__ CUtensorMap tm_xl,
           const __grid_constant__ CUtensorMap tm_wh, const __grid_constant__ CUtensorMap tm_wl,
           const BFit *__restrict__ fits, const BState *__restrict__ state, const EItem *__restrict__ items,
           int nitems, const float *__restrict__ bias, const float *__restrict__ chi, const float *__restrict__ clo,
           double *__restrict__ epart, int *err) {
  using namespace tc;
  extern __shared__ uint8_t smem_raw[];
  BTSmem &S = smem_aligned<BTSmem>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < 2; s++) mbar_init(&S.x_full[s], 1), mbar_init(&S.x_empty[s], 1);
    for (int s = 0; s < kTWS; s++) mbar_init(&S.w_full[s], 1), mbar_init(&S.w_empty[s], 1);
    for (int s = 0; s < 2; s++) mbar_init(&S.acc_full[s], 1), mbar_init(&S.acc_empty[s], 4);
    mbar_init(&S.mma_done, 1);
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&S.tmem_base, 256);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tmem_base;
  // every role walks the same (item, tile, group) sequence
  if (warp == 0) {
    if (elect_one()) {
      uint32_t xi = 0, wi = 0;
      bool ok = true;
      for (int ii = blockIdx.x; ii < nitems && ok; ii += gridDim.x) {
        const EItem it = items[ii];
        if (!state[it.fit].active) continue;
        const BFit &F = fits[it.fit];
        const int ntile = (int)min((int64_t)4, (F.n - it.p0 + kTT - 1) / kTT), G = (F.k + 3) / 4;
        for (int t = 0; t < ntile && ok; t++) {
          const int xb = xi & 1;
          if (!(ok = mbar_wait(&S.x_empty[xb], ((xi >> 1) & 1) ^ 1, err))) break;
          mbar_expect_tx(&S.x_full[xb], 2 * kTT * 128);
          const int row = (int)(F.xrow + it.p0 + (int64_t)kTT * t);
          tma_load_2d(S.xh[xb], &tm_xh, &S.x_full[xb], 0, row);
          tma_load_2d(S.xl[xb], &tm_xl, &S.x_full[xb], 0, row);
          xi++;
          for (int g = 0; g < G; g++) {
            const int ws = wi % kTWS;
            if (!(ok = mbar_wait(&S.w_empty[ws], ((wi / kTWS) & 1) ^ 1, err))) break;
            mbar_expect_tx(&S.w_full[ws], 2 * 128 * 128);
            tma_load_2d(S.wh[ws], &tm_wh, &S.w_full[ws], 0, (F.wg + g) * 128);
            tma_load_2d(S.wl[ws], &tm_wl, &S.w_full[ws], 0, (F.wg + g) * 128);
            wi++;
          }
        }
      }
      for (int s = 0; s < 2 && xi > (uint32_t)s; s++) {
        const uint32_t u = xi - 1 - s;
        mbar_wait_drain(&S.x_full[u & 1], (u >> 1) & 1);
      }
      for (int s = 0; s < kTWS && wi > (uint32_t)s; s++) {
        const uint32_t u = wi - 1 - s;
        mbar_wait_drain(&S.w_full[u % kTWS], (u / kTWS) & 1);
      }
    }
  } else if (warp == 1) {
    if (elect_one()) {
      uint32_t xi = 0, wi = 0, ai = 0;
      bool ok = true;
      for (int ii = blockIdx.x; ii < nitems && ok; ii += gridDim.x) {
        const EItem it = items[ii];
        if (!state[it.fit].active) continue;
        const BFit &F = fits[it.fit];
        const int ntile = (int)min((int64_t)4, (F.n - it.p0 + kTT - 1) / kTT), G = (F.k + 3) / 4;
        for (int t = 0; t < ntile && ok; t++) {
          const int xb = xi & 1;
          if (!(ok = mbar_wait(&S.x_full[xb], (xi >> 1) & 1, err))) break;
          tc_fence_after();
          const uint64_t dxh = sdesc_sw128(smem_u32(S.xh[xb])), dxl = sdesc_sw128(smem_u32(S.xl[xb]));
          for (int g = 0; g < G && ok; g++) {
            const int ws = wi % kTWS, ab = ai & 1;
            if (!(ok = mbar_wait(&S.w_full[ws], (wi / kTWS) & 1, err))) break;
            if (!(ok = mbar_wait(&S.acc_empty[ab], ((ai >> 1) & 1) ^ 1, err))) break;
            tc_fence_after();
            const uint64_t dwh = sdesc_sw128(smem_u32(S.wh[ws])), dwl = sdesc_sw128(smem_u32(S.wl[ws]));
            const uint32_t dt = tbase + ab * 128;
            // the small cross products first, x_h W_h last
#pragma unroll
            for (int p = 0; p < 3; p++) {
              const uint64_t da = (p == 1) ? dxl : dxh;
              const uint64_t db = (p == 0) ? dwl : dwh;
#pragma unroll
              for (int kb = 0; kb < 2; kb++)
                mma_f16(dt, da + 2 * kb, db + 2 * kb, idesc_f16(kTT, kb ? 64 : 128), (p | kb) != 0);
            }
            mma_commit(&S.acc_full[ab]);
            mma_commit(&S.w_empty[ws]);
            wi++;
            ai++;
          }
          if (!ok) break;
          mma_commit(&S.x_empty[xb]);
          xi++;
        }
      }
      mma_commit(&S.mma_done);
      mbar_wait_drain(&S.mma_done, 0);
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 = points of the tile
    const int quad = warp & 3, row = quad * 32 + lane;
    const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
    uint32_t ai = 0;
    int icnt = 0;
    bool ok = true;
    for (int ii = blockIdx.x; ii < nitems && ok; ii += gridDim.x) {
      const EItem it = items[ii];
      if (!state[it.fit].active) continue;
      const BFit &F = fits[it.fit];
      const int64_t n = F.n;
      const int K = F.k, G = (K + 3) / 4;
      const int ntile = (int)min((int64_t)4, (n - it.p0 + kTT - 1) / kTT);
      double lsum = 0.0;
      for (int t = 0; t < ntile && ok; t++) {
        const int64_t i = it.p0 + (int64_t)kTT * t + row;
        const bool valid = i < n;
        float mx = -INFINITY, se = 0.f;
        for (int g = 0; g < G; g++) {
          const int ab = ai & 1;
          if (!(ok = mbar_wait_warp(&S.acc_full[ab], (ai >> 1) & 1, err))) break;
          tc_fence_after();
          uint32_t v[128];
          tmem_ld64(tbase + lane_addr + ab * 128, *reinterpret_cast<uint32_t(*)[64]>(v));
          tmem_ld64(tbase + lane_addr + ab * 128 + 64, *reinterpret_cast<uint32_t(*)[64]>(v + 64));
          tmem_wait_ld();
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&S.acc_empty[ab]);
          ai++;
          const float *bg = bias + (size_t)(F.wg + g) * 128;
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const int j = 4 * g + q;
            float s0 = 0.f, s1 = 0.f;
#pragma unroll
            for (int u = 0; u < 16; u += 4) {
              const float4 b0 = __ldg(reinterpret_cast<const float4 *>(bg + 16 * q + u));
              const float4 b1 = __ldg(reinterpret_cast<const float4 *>(bg + 64 + 16 * q + u));
              const float a0 = __uint_as_float(v[16 * q + u]) - b0.x, a1 = __uint_as_float(v[16 * q + u + 1]) - b0.y;
              const float a2 = __uint_as_float(v[16 * q + u + 2]) - b0.z, a3 = __uint_as_float(v[16 * q + u + 3]) - b0.w;
              const float c0 = __uint_as_float(v[64 + 16 * q + u]) - b1.x;
              const float c1 = __uint_as_float(v[64 + 16 * q + u + 1]) - b1.y;
              const float c2 = __uint_as_float(v[64 + 16 * q + u + 2]) - b1.z;
              const float c3 = __uint_as_float(v[64 + 16 * q + u + 3]) - b1.w;
              s0 = fmaf(a0, a0, fmaf(a1, a1, fmaf(a2, a2, fmaf(a3, a3, s0))));
              s1 = fmaf(c0, c0, fmaf(c1, c1, fmaf(c2, c2, fmaf(c3, c3, s1))));
            }
            if (j < K) {
              const float l = (chi[(size_t)(F.wg + g) * 4 + q] - 0.5f * (s0 + s1)) + clo[(size_t)(F.wg + g) * 4 + q];
              if (valid) F.R[(size_t)j * n + i] = l;
              blse_push(l, mx, se);
            }
          }
        }
        if (!ok) break;
        const float lse = mx + logf(se);
        if (valid) {
          lsum += (double)lse;
          for (int j = 0; j < K; j++) F.R[(size_t)j * n + i] = expf(F.R[(size_t)j * n + i] - lse);
        }
      }
      // the item's LogL partial, summed in a fixed order over the 4 warps
      const int par = icnt++ & 1;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
      if (lane == 0) S.red[par][warp - 2] = lsum;
      // the four warps leave together when a wait gave up
      if (!(ok = bar_and(1, 128, ok))) break;
      if (threadIdx.x == 64) epart[ii] = ((S.red[par][0] + S.red[par][1]) + S.red[par][2]) + S.red[par][3];
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tbase, 256);
}
}  // namespace
}  // namespace fem

using namespace fem;

struct fem_em_batch {
  int nfits = 0;
  fem_em_config cfg{};
  cudaStream_t stream = nullptr;
  std::vector<BFit> hfits;
  std::vector<char> have_data, have_params;
  int cap = 0;                      // trace entries per fit
  // device
  BFit *fits = nullptr;
  BState *state = nullptr;
  float *X = nullptr, *R = nullptr, *muT = nullptr, *WT = nullptr, *logcT = nullptr;
  double *pi = nullptr, *mu = nullptr, *sigma = nullptr, *psum = nullptr, *logc = nullptr;
  double *epart = nullptr, *mpart = nullptr, *cpart = nullptr;
  double *trace = nullptr, *etrace = nullptr;
  int *nactive = nullptr, *hnactive = nullptr;   // device / pinned host
  EItem *eitems = nullptr;
  MItem *mitems = nullptr;
  CItem *citems = nullptr;
  int2 *comps = nullptr;
  int ncomps = 0;
  int e_beg[kClasses + 1] = {}, m_beg[kClasses + 1] = {}, c_beg[kClasses + 1] = {};
  size_t c_smem[kClasses] = {};
  int c_kmax[kClasses] = {};       // largest k of the class's fits
  size_t m_smem[kClasses] = {};     // means kernel dynamic shared memory
  fem_em_batch_tuning tuning{};     // work-item sizes per class
  // mixed form: tensor-core E-step of the d <= 32 class
  bool tc = false;
  int tc_nfits = 0, tc_groups = 0, tc_grid = 0;
  int64_t tc_rows = 0;
  int *tfits = nullptr;             // the class's fits
  int2 *tgroups = nullptr;          // (fit, group) per W group
  __half *Xh = nullptr, *Xl = nullptr, *Wh = nullptr, *Wl = nullptr;
  float *tbias = nullptr, *tchi = nullptr, *tclo = nullptr;
  int *terr = nullptr;              // bounded-wait status of the tensor-core kernel
  CUtensorMap tm_xh{}, tm_xl{}, tm_wh{}, tm_wl{};
  std::vector<BState> hstate;
  // timing: phase boundaries of the sweeps since the last host sync
  bool timing = false;
  cudaEvent_t pev[kBatchSyncEvery][kTimeMarks] = {};
  cudaEvent_t ev_start = nullptr, ev_end = nullptr;
  double t_phase[5] = {};           // E-step, means, covariance, factorisation, whole sweep loop
  double t_class[3][kClasses] = {}; // E-step, means, covariance launches per dimension class
  int64_t launches = 0, sweeps = 0;
};

namespace {

int check_batch(fem_em_batch *b) {
  if (!b) {
    set_error("null batch handle");
    return FEM_ERR_BAD_ARG;
  }
  return FEM_OK;
}

int check_fit(fem_em_batch *b, int fit) {
  FEM_TRY(check_batch(b));
  if (fit < 0 || fit >= b->nfits) {
    set_error("fit index %d out of range [0, %d)", fit, b->nfits);
    return FEM_ERR_BAD_ARG;
  }
  return FEM_OK;
}

void free_batch(fem_em_batch *b) {
  dfree(b->fits);
  dfree(b->state);
  dfree(b->X);
  dfree(b->R);
  dfree(b->muT);
  dfree(b->WT);
  dfree(b->logcT);
  dfree(b->pi);
  dfree(b->mu);
  dfree(b->sigma);
  dfree(b->psum);
  dfree(b->logc);
  dfree(b->epart);
  dfree(b->mpart);
  dfree(b->cpart);
  dfree(b->trace);
  dfree(b->etrace);
  dfree(b->nactive);
  dfree(b->eitems);
  dfree(b->mitems);
  dfree(b->citems);
  dfree(b->comps);
  dfree(b->tfits);
  dfree(b->tgroups);
  dfree(b->Xh);
  dfree(b->Xl);
  dfree(b->Wh);
  dfree(b->Wl);
  dfree(b->tbias);
  dfree(b->tchi);
  dfree(b->tclo);
  dfree(b->terr);
  if (b->hnactive) cudaFreeHost(b->hnactive);
  for (auto &row : b->pev)
    for (auto &e : row)
      if (e) cudaEventDestroy(e);
  if (b->ev_start) cudaEventDestroy(b->ev_start);
  if (b->ev_end) cudaEventDestroy(b->ev_end);
  if (b->stream) cudaStreamDestroy(b->stream);
}

template <class T>
int upload_vec(T **dst, const std::vector<T> &v) {
  FEM_TRY(dalloc(dst, v.size()));
  if (!v.empty()) FEM_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return FEM_OK;
}


void mark(fem_em_batch *b, int slot, int m) {
  if (b->timing) cudaEventRecord(b->pev[slot][m], b->stream);
}

// device time of the sweeps recorded in event slots [0, pending); marks: 0 sweep
// start, 1..4 after each class's E-step, 5..8 after each class's means, 9 after
// their reduction, 10..13 after each class's covariance sums, 14 sweep end
void collect_timing(fem_em_batch *b, int pending) {
  float ms = 0.f;
  for (int s = 0; s < pending; s++) {
    const cudaEvent_t *e = b->pev[s];
    const int bounds[5] = {0, 4, 9, 13, 14};
    for (int p = 0; p < 4; p++)
      if (cudaEventElapsedTime(&ms, e[bounds[p]], e[bounds[p + 1]]) == cudaSuccess) b->t_phase[p] += ms;
    for (int c = 0; c < kClasses; c++) {
      if (cudaEventElapsedTime(&ms, e[c], e[1 + c]) == cudaSuccess) b->t_class[0][c] += ms;
      if (cudaEventElapsedTime(&ms, e[4 + c], e[5 + c]) == cudaSuccess) b->t_class[1][c] += ms;
      if (cudaEventElapsedTime(&ms, e[9 + c], e[10 + c]) == cudaSuccess) b->t_class[2][c] += ms;
    }
  }
}

// tensor-core operands of the d <= 32 class from the factorisation just enqueued
int prep_tc(fem_em_batch *b) {
  if (!b->tc) return FEM_OK;
  k_bt_prep<<<b->tc_groups, 128, 0, b->stream>>>(b->fits, b->tgroups, b->Wh, b->Wl, b->tbias, b->tchi, b->tclo);
  FEM_CUDA(cudaGetLastError());
  b->launches++;
  return FEM_OK;
}

int launch_sweep(fem_em_batch *b, int it, int svd, int slot) {
  const BFit *fits = b->fits;
  BState *st = b->state;
  mark(b, slot, 0);
  for (int c = 0; c < kClasses; c++) {
    const int cnt = b->e_beg[c + 1] - b->e_beg[c];
    if (!cnt) {
      mark(b, slot, 1 + c);
      continue;
    }
    const EItem *it0 = b->eitems + b->e_beg[c];
    double *ep = b->epart + b->e_beg[c];
    if (c == kTClass && b->tc) {
      k_bt_estep<<<std::min(b->tc_grid, cnt), kTThreads, sizeof(BTSmem) + 1024, b->stream>>>(
          b->tm_xh, b->tm_xl, b->tm_wh, b->tm_wl, fits, st, it0, cnt, b->tbias, b->tchi, b->tclo, ep, b->terr);
      FEM_CUDA(cudaGetLastError());
      b->launches++;
      mark(b, slot, 1 + c);
      continue;
    }
    switch (c) {
      case 0: k_b_estep<4, kBEP><<<cnt, kBEThreads, estep_smem<4>(), b->stream>>>(fits, st, it0, ep); break;
      case 1: k_b_estep<8, kBEP><<<cnt, kBEThreads, estep_smem<8>(), b->stream>>>(fits, st, it0, ep); break;
      case 2: k_b_estep<16, kBEP><<<cnt, kBEThreads, estep_smem<16>(), b->stream>>>(fits, st, it0, ep); break;
      default: k_b_estep<32, kBEP><<<cnt, kBEThreads, estep_smem<32>(), b->stream>>>(fits, st, it0, ep); break;
    }
    FEM_CUDA(cudaGetLastError());
    b->launches++;
    mark(b, slot, 1 + c);
  }
  for (int c = 0; c < kClasses; c++) {
    const int cnt = b->m_beg[c + 1] - b->m_beg[c];
    if (!cnt) {
      mark(b, slot, 5 + c);
      continue;
    }
    const MItem *it0 = b->mitems + b->m_beg[c];
    switch (c) {
      case 0: k_b_means<4><<<cnt, kBMThreads, b->m_smem[c], b->stream>>>(fits, st, it0, b->mpart, b->c_kmax[c]); break;
      case 1: k_b_means<8><<<cnt, kBMThreads, b->m_smem[c], b->stream>>>(fits, st, it0, b->mpart, b->c_kmax[c]); break;
      case 2: k_b_means<16><<<cnt, kBMThreads, b->m_smem[c], b->stream>>>(fits, st, it0, b->mpart, b->c_kmax[c]); break;
      default: k_b_means<32><<<cnt, kBMThreads, b->m_smem[c], b->stream>>>(fits, st, it0, b->mpart, b->c_kmax[c]); break;
    }
    FEM_CUDA(cudaGetLastError());
    b->launches++;
    mark(b, slot, 5 + c);
  }
  k_b_final_means<128><<<b->nfits, 128, 0, b->stream>>>(fits, st, b->epart, b->mpart);
  FEM_CUDA(cudaGetLastError());
  b->launches++;
  mark(b, slot, 9);
  for (int c = 0; c < kClasses; c++) {
    const int cnt = b->c_beg[c + 1] - b->c_beg[c];
    if (!cnt) {
      mark(b, slot, 10 + c);
      continue;
    }
    const CItem *it0 = b->citems + b->c_beg[c];
    const size_t sm = b->c_smem[c];
    switch (c) {
      case 0: k_b_cov_own<4><<<cnt, kBCThreads, sm, b->stream>>>(fits, st, it0, b->cpart, b->c_kmax[c]); break;
      case 1: k_b_cov_own<8><<<cnt, kBCThreads, sm, b->stream>>>(fits, st, it0, b->cpart, b->c_kmax[c]); break;
      case 2: k_b_cov_own<16><<<cnt, kBCThreads, sm, b->stream>>>(fits, st, it0, b->cpart, b->c_kmax[c]); break;
      default: k_b_cov<32><<<cnt, kBCThreads, sm, b->stream>>>(fits, st, it0, b->cpart); break;
    }
    FEM_CUDA(cudaGetLastError());
    b->launches++;
    mark(b, slot, 10 + c);
  }
  k_b_factor<<<b->ncomps, kBFThreads, 0, b->stream>>>(fits, st, b->comps, b->cpart, b->cfg.reg_coef, 1, svd);
  FEM_CUDA(cudaGetLastError());
  FEM_TRY(prep_tc(b));
  k_b_sweep_end<<<1, 1024, 0, b->stream>>>(st, b->nfits, it, b->cfg.max_sweeps, b->cfg.eps, b->cfg.abort_thr, svd,
                                           b->trace, b->etrace, b->cap, b->nactive);
  FEM_CUDA(cudaGetLastError());
  b->launches += 2;
  mark(b, slot, 14);
  return FEM_OK;
}

}  // namespace

extern "C" void fem_em_batch_tuning_default(fem_em_batch_tuning *t) {
  if (!t) return;
  for (int c = 0; c < kClasses; c++) t->means_chunk[c] = kBMChunk, t->cov_chunk[c] = kBCChunk;
}

extern "C" int fem_em_batch_create(int nfits, const int *d, const int64_t *n, const int *k,
                                   const fem_em_config *cfg, fem_em_batch **out) {
  return fem_em_batch_create_tuned(nfits, d, n, k, cfg, nullptr, out);
}

extern "C" int fem_em_batch_create_tuned(int nfits, const int *d, const int64_t *n, const int *k,
                                         const fem_em_config *cfg, const fem_em_batch_tuning *tuning,
                                         fem_em_batch **out) {
  if (!out || nfits < 1 || !d || !n || !k) {
    set_error("fem_em_batch_create: bad arguments");
    return FEM_ERR_BAD_ARG;
  }
  *out = nullptr;
  fem_em_batch_tuning tune;
  fem_em_batch_tuning_default(&tune);
  if (tuning) tune = *tuning;
  for (int c = 0; c < kClasses; c++) {
    const int a = tune.means_chunk[c], v = tune.cov_chunk[c];
    if (a < 256 || a > 16384 || a % 128 || v < 256 || v > 16384 || v % 128) {
      set_error("tuning: class %d item sizes must be multiples of 128 in [256, 16384] (means %d, cov %d)", c, a, v);
      return FEM_ERR_BAD_ARG;
    }
  }
  fem_em_config c;
  if (cfg) c = *cfg;
  else {
    fem_em_config_default(&c);
    c.precision = FEM_PREC_FP32;
  }
  if (c.precision != FEM_PREC_FP32 && c.precision != FEM_PREC_MIXED) {
    set_error("batched fits run in FP32 (FEM_PREC_FP32) or with the tensor-core E-step for d > 16 (FEM_PREC_MIXED)");
    return FEM_ERR_UNSUPPORTED;
  }
  if (c.max_sweeps < 1) {
    set_error("max_sweeps must be >= 1");
    return FEM_ERR_BAD_ARG;
  }
  for (int f = 0; f < nfits; f++) {
    if (d[f] < 1 || k[f] < 1 || n[f] < 1) {
      set_error("fit %d: d, n and k must be positive", f);
      return FEM_ERR_BAD_ARG;
    }
    if (d[f] > kBMaxD || k[f] > kBMaxK || n[f] >= ((int64_t)1 << 31)) {
      set_error("fit %d: batched fits need d <= %d, k <= %d, n < 2^31 (got d=%d k=%d n=%lld)", f, kBMaxD,
                kBMaxK, d[f], k[f], (long long)n[f]);
      return FEM_ERR_UNSUPPORTED;
    }
  }
  FEM_TRY(select_device(c.device));
  fem_em_batch *b = new (std::nothrow) fem_em_batch;
  if (!b) {
    set_error("out of host memory");
    return FEM_ERR_BAD_ARG;
  }
  b->nfits = nfits;
  b->cfg = c;
  b->tuning = tune;
  b->hfits.resize(nfits);
  b->have_data.assign(nfits, 0);
  b->have_params.assign(nfits, 0);
  b->cap = std::min(c.max_sweeps, 4096);
  int st = FEM_OK;
  auto fail = [&](int s) {
    free_batch(b);
    delete b;
    return s;
  };
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("stream creation failed");
    return fail(FEM_ERR_CUDA);
  }
  // sizes and offsets
  int64_t nx = 0, nr = 0, nk = 0, nkd = 0, nkdd = 0, nkD = 0, nkT = 0;
  std::vector<int64_t> ox(nfits), orr(nfits), ok_(nfits), okd(nfits), okdd(nfits), okD(nfits), okT(nfits);
  for (int f = 0; f < nfits; f++) {
    const int D = class_dim(class_of(d[f]));
    ox[f] = nx, orr[f] = nr, ok_[f] = nk, okd[f] = nkd, okdd[f] = nkdd, okD[f] = nkD, okT[f] = nkT;
    nx += (n[f] * d[f] + 3) & ~(int64_t)3;
    nr += n[f] * k[f];
    nk += k[f];
    nkd += (int64_t)k[f] * d[f];
    nkdd += (int64_t)k[f] * d[f] * d[f];
    nkD += (int64_t)k[f] * D;
    nkT += (int64_t)k[f] * tri_off(D);
  }
  if ((st = dalloc(&b->X, nx)) || (st = dalloc(&b->R, nr)) || (st = dalloc(&b->muT, nkD)) ||
      (st = dalloc(&b->WT, nkT)) || (st = dalloc(&b->logcT, nk)) || (st = dalloc(&b->pi, nk)) ||
      (st = dalloc(&b->mu, nkd)) || (st = dalloc(&b->sigma, nkdd)) || (st = dalloc(&b->psum, nk)) ||
      (st = dalloc(&b->logc, nk)))
    return fail(st);
  // work items, grouped by dimension class
  std::vector<EItem> ei;
  std::vector<MItem> mi;
  std::vector<CItem> ci;
  std::vector<int2> comps, tgroups;
  std::vector<int> tfits;
  int64_t mp = 0, cp = 0;
  for (int f = 0; f < nfits; f++) {
    BFit &F = b->hfits[f];
    F.X = b->X + ox[f];
    F.R = b->R + orr[f];
    F.n = n[f];
    F.d = d[f];
    F.k = k[f];
    F.D = class_dim(class_of(d[f]));
    F.pi = b->pi + ok_[f];
    F.mu = b->mu + okd[f];
    F.sigma = b->sigma + okdd[f];
    F.psum = b->psum + ok_[f];
    F.logc = b->logc + ok_[f];
    F.muT = b->muT + okD[f];
    F.WT = b->WT + okT[f];
    F.logcT = b->logcT + ok_[f];
    F.xrow = -1;
    F.wg = 0;
    if (c.precision == FEM_PREC_MIXED && class_of(d[f]) == kTClass) {
      F.xrow = b->tc_rows;
      F.wg = b->tc_groups;
      b->tc_rows += n[f];
      for (int g = 0; g < (k[f] + 3) / 4; g++) tgroups.push_back(make_int2(f, g));
      b->tc_groups += (k[f] + 3) / 4;
      tfits.push_back(f);
    }
    for (int j = 0; j < k[f]; j++) comps.push_back(make_int2(f, j));
  }
  for (int c = 0; c < kClasses; c++) {
    b->e_beg[c] = (int)ei.size();
    b->m_beg[c] = (int)mi.size();
    b->c_beg[c] = (int)ci.size();
    int kmax = 0;
    for (int f = 0; f < nfits; f++) {
      BFit &F = b->hfits[f];
      if (class_of(F.d) != c) continue;
      kmax = std::max(kmax, F.k);
      const int ep = kBEPoints;
      F.e_first = (int)ei.size();
      for (int64_t p = 0; p < F.n; p += ep) ei.push_back(EItem{f, (int)p});
      F.e_count = (int)ei.size() - F.e_first;
      F.m_first = (int)mi.size();
      F.m_part = mp;
      const int mch = tune.means_chunk[c], cch = tune.cov_chunk[c];
      for (int64_t p = 0; p < F.n; p += mch) {
        mi.push_back(MItem{f, (int)p, (int)std::min<int64_t>(F.n, p + mch), mp});
        mp += (int64_t)F.k * (F.D + 4);
      }
      F.m_count = (int)mi.size() - F.m_first;
      F.nug = class_owner(F.D) ? 1 : (F.k * class_nblk(F.D) + 255) / 256;
      F.c_part = cp;
      F.c_stride = 0;
      for (int ug = 0; ug < F.nug; ug++) {
        int u0, u1, ng, per;
        unit_range(F.k, F.D, ug, &u0, &u1, &ng, &per);
        F.c_stride += (int64_t)ng * (u1 - u0) * per;
      }
      F.c_chunks = 0;
      for (int64_t p = 0; p < F.n; p += cch) {
        int64_t off = cp;
        for (int ug = 0; ug < F.nug; ug++) {
          int u0, u1, ng, per;
          unit_range(F.k, F.D, ug, &u0, &u1, &ng, &per);
          ci.push_back(CItem{f, (int)p, (int)std::min<int64_t>(F.n, p + cch), u0, u1, off});
          off += (int64_t)ng * (u1 - u0) * per;
        }
        cp += F.c_stride;
        F.c_chunks++;
      }
    }
    const int D = class_dim(c), nblk = class_nblk(D);
    const int cj = std::max(1, std::min(kmax, 256 / nblk + 2));
    b->c_kmax[c] = std::max(kmax, 1);
    {
      size_t mf = 0;
      switch (c) {
        case 0: mf = means_buf_floats<4>(b->c_kmax[c]); break;
        case 1: mf = means_buf_floats<8>(b->c_kmax[c]); break;
        case 2: mf = means_buf_floats<16>(b->c_kmax[c]); break;
        default: mf = means_buf_floats<32>(b->c_kmax[c]); break;
      }
      // two tile buffers; the point-group reduction reuses them (<= 128 x 16 floats)
      b->m_smem[c] = std::max<size_t>(2 * mf, (size_t)kBMThreads * 16) * sizeof(float);
    }
    b->c_smem[c] = (class_owner(D) ? 2 * own_buf_floats(D, b->c_kmax[c]) : CovGeom<32>::floats(cj)) * sizeof(float);
  }
  b->e_beg[kClasses] = (int)ei.size();
  b->m_beg[kClasses] = (int)mi.size();
  b->c_beg[kClasses] = (int)ci.size();
  b->ncomps = (int)comps.size();
  if ((st = upload_vec(&b->eitems, ei)) || (st = upload_vec(&b->mitems, mi)) || (st = upload_vec(&b->citems, ci)) ||
      (st = upload_vec(&b->comps, comps)) || (st = dalloc(&b->epart, ei.size())) || (st = dalloc(&b->mpart, mp)) ||
      (st = dalloc(&b->cpart, cp)) || (st = dalloc(&b->state, nfits)) ||
      (st = dalloc(&b->trace, (size_t)nfits * b->cap)) || (st = dalloc(&b->etrace, (size_t)nfits * b->cap)) ||
      (st = dalloc(&b->nactive, 1)) || (st = upload_vec(&b->fits, b->hfits)))
    return fail(st);
  if (!tfits.empty()) {
    b->tc = true;
    b->tc_nfits = (int)tfits.size();
    b->tc_grid = sm_count();
    if ((st = upload_vec(&b->tfits, tfits)) || (st = upload_vec(&b->tgroups, tgroups)) ||
        (st = dalloc(&b->Xh, (size_t)b->tc_rows * 64)) || (st = dalloc(&b->Xl, (size_t)b->tc_rows * 64)) ||
        (st = dalloc(&b->Wh, (size_t)b->tc_groups * 128 * 64)) || (st = dalloc(&b->Wl, (size_t)b->tc_groups * 128 * 64)) ||
        (st = dalloc(&b->tbias, (size_t)b->tc_groups * 128)) || (st = dalloc(&b->tchi, (size_t)b->tc_groups * 4)) ||
        (st = dalloc(&b->tclo, (size_t)b->tc_groups * 4)) || (st = dalloc(&b->terr, 1)))
      return fail(st);
    if ((st = encode_tmap_2d(&b->tm_xh, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, b->Xh, 64, (uint64_t)b->tc_rows, 64, kTT,
                             CU_TENSOR_MAP_SWIZZLE_128B, 128)) ||
        (st = encode_tmap_2d(&b->tm_xl, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, b->Xl, 64, (uint64_t)b->tc_rows, 64, kTT,
                             CU_TENSOR_MAP_SWIZZLE_128B, 128)) ||
        (st = encode_tmap_2d(&b->tm_wh, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, b->Wh, 64, (uint64_t)b->tc_groups * 128, 64,
                             128, CU_TENSOR_MAP_SWIZZLE_128B, 128)) ||
        (st = encode_tmap_2d(&b->tm_wl, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, b->Wl, 64, (uint64_t)b->tc_groups * 128, 64,
                             128, CU_TENSOR_MAP_SWIZZLE_128B, 128)))
      return fail(st);
    if (cudaFuncSetAttribute(k_bt_estep, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(BTSmem) + 1024)) != cudaSuccess) {
      set_error("tensor-core E-step shared-memory limit could not be raised");
      return fail(FEM_ERR_CUDA);
    }
  }
  if (cudaMallocHost((void **)&b->hnactive, sizeof(int)) != cudaSuccess) {
    set_error("pinned allocation failed");
    return fail(FEM_ERR_CUDA);
  }
  for (auto &row : b->pev)
    for (auto &e : row)
      if (cudaEventCreate(&e) != cudaSuccess) {
        set_error("event creation failed");
        return fail(FEM_ERR_CUDA);
      }
  if (cudaEventCreate(&b->ev_start) != cudaSuccess || cudaEventCreate(&b->ev_end) != cudaSuccess) {
    set_error("event creation failed");
    return fail(FEM_ERR_CUDA);
  }
  if (allow_dyn_smem(k_b_estep<4, kBEP>, estep_smem<4>()) != cudaSuccess ||
      allow_dyn_smem(k_b_estep<8, kBEP>, estep_smem<8>()) != cudaSuccess ||
      allow_dyn_smem(k_b_estep<16, kBEP>, estep_smem<16>()) != cudaSuccess ||
      allow_dyn_smem(k_b_estep<32, kBEP>, estep_smem<32>()) != cudaSuccess ||
      allow_dyn_smem(k_b_means<4>, b->m_smem[0]) != cudaSuccess ||
      allow_dyn_smem(k_b_means<8>, b->m_smem[1]) != cudaSuccess ||
      allow_dyn_smem(k_b_means<16>, b->m_smem[2]) != cudaSuccess ||
      allow_dyn_smem(k_b_means<32>, b->m_smem[3]) != cudaSuccess ||
      allow_dyn_smem(k_b_cov_own<4>, b->c_smem[0]) != cudaSuccess ||
      allow_dyn_smem(k_b_cov_own<8>, b->c_smem[1]) != cudaSuccess ||
      allow_dyn_smem(k_b_cov_own<16>, b->c_smem[2]) != cudaSuccess ||
      allow_dyn_smem(k_b_cov<32>, b->c_smem[3]) != cudaSuccess) {
    set_error("batched kernels' shared-memory limits could not be raised");
    return fail(FEM_ERR_CUDA);
  }
  b->hstate.resize(nfits);
  *out = b;
  return FEM_OK;
}

extern "C" void fem_em_batch_destroy(fem_em_batch *b) {
  if (!b) return;
  cudaSetDevice(b->cfg.device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  free_batch(b);
  delete b;
}

extern "C" int fem_em_batch_upload(fem_em_batch *b, int fit, const float *X, int64_t ld) {
  FEM_TRY(check_fit(b, fit));
  const BFit &F = b->hfits[fit];
  if (!X || ld < F.d) {
    set_error("fem_em_batch_upload: null rows or ld < d");
    return FEM_ERR_BAD_ARG;
  }
  FEM_CUDA(cudaSetDevice(b->cfg.device));
  FEM_CUDA(cudaMemcpy2DAsync((void *)F.X, (size_t)F.d * sizeof(float), X, (size_t)ld * sizeof(float),
                             (size_t)F.d * sizeof(float), (size_t)F.n, cudaMemcpyHostToDevice, b->stream));
  FEM_CUDA(cudaStreamSynchronize(b->stream));
  b->have_data[fit] = 1;
  return FEM_OK;
}

extern "C" int fem_em_batch_upload_packed(fem_em_batch *b, const float *X) {
  FEM_TRY(check_batch(b));
  if (!X) {
    set_error("fem_em_batch_upload_packed: null rows");
    return FEM_ERR_BAD_ARG;
  }
  FEM_CUDA(cudaSetDevice(b->cfg.device));
  const float *src = X;
  for (int f = 0; f < b->nfits; f++) {
    const BFit &F = b->hfits[f];
    FEM_CUDA(cudaMemcpyAsync((void *)F.X, src, (size_t)F.n * F.d * sizeof(float), cudaMemcpyHostToDevice,
                             b->stream));
    src += (size_t)F.n * F.d;
    b->have_data[f] = 1;
  }
  FEM_CUDA(cudaStreamSynchronize(b->stream));
  return FEM_OK;
}

extern "C" int fem_em_batch_set_params(fem_em_batch *b, int fit, const double *pi, const double *mu,
                                       const double *sigma) {
  FEM_TRY(check_fit(b, fit));
  if (!pi || !mu || !sigma) {
    set_error("fem_em_batch_set_params: null argument");
    return FEM_ERR_BAD_ARG;
  }
  const BFit &F = b->hfits[fit];
  const int k = F.k, d = F.d, D = F.D;
  std::vector<float> muT((size_t)k * D, 0.f);
  for (int j = 0; j < k; j++)
    for (int q = 0; q < d; q++) muT[(size_t)j * D + q] = (float)mu[(size_t)j * d + q];
  FEM_CUDA(cudaSetDevice(b->cfg.device));
  FEM_CUDA(cudaMemcpyAsync(F.pi, pi, (size_t)k * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  FEM_CUDA(cudaMemcpyAsync(F.mu, mu, (size_t)k * d * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  FEM_CUDA(cudaMemcpyAsync(F.sigma, sigma, (size_t)k * d * d * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  FEM_CUDA(cudaMemcpyAsync(F.muT, muT.data(), muT.size() * sizeof(float), cudaMemcpyHostToDevice, b->stream));
  FEM_CUDA(cudaStreamSynchronize(b->stream));
  b->have_params[fit] = 1;
  return FEM_OK;
}

extern "C" int fem_em_batch_get_params(fem_em_batch *b, int fit, double *pi, double *mu, double *sigma) {
  FEM_TRY(check_fit(b, fit));
  const BFit &F = b->hfits[fit];
  FEM_CUDA(cudaSetDevice(b->cfg.device));
  if (pi) FEM_CUDA(cudaMemcpyAsync(pi, F.pi, (size_t)F.k * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (mu)
    FEM_CUDA(cudaMemcpyAsync(mu, F.mu, (size_t)F.k * F.d * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (sigma)
    FEM_CUDA(cudaMemcpyAsync(sigma, F.sigma, (size_t)F.k * F.d * F.d * sizeof(double), cudaMemcpyDeviceToHost,
                             b->stream));
  FEM_CUDA(cudaStreamSynchronize(b->stream));
  return FEM_OK;
}

extern "C" int fem_em_batch_set_parameters(fem_em_batch *b, int max_sweeps, double eps, double abort_thr,
                                           double reg_coef) {
  FEM_TRY(check_batch(b));
  if (max_sweeps < 1) {
    set_error("max_sweeps must be >= 1");
    return FEM_ERR_BAD_ARG;
  }
  b->cfg.max_sweeps = max_sweeps;
  b->cfg.eps = eps;
  b->cfg.abort_thr = abort_thr;
  b->cfg.reg_coef = reg_coef;
  return FEM_OK;
}

extern "C" int fem_em_batch_train(fem_em_batch *b, int svd, int *status, int *iter_counter, double *logl) {
  FEM_TRY(check_batch(b));
  for (int f = 0; f < b->nfits; f++)
    if (!b->have_data[f] || !b->have_params[f]) {
      set_error("fit %d: train needs an uploaded dataset and parameters", f);
      return FEM_ERR_STATE;
    }
  FEM_CUDA(cudaSetDevice(b->cfg.device));
  for (auto &s : b->hstate) {
    s = BState{};
    s.active = 1;
    s.status = FEM_OK;
    s.chol_failed = INT_MAX;
    s.prev = -DBL_MAX;
    s.logl = -DBL_MAX;
    s.fail_comp = -1;
  }
  FEM_CUDA(cudaMemcpyAsync(b->state, b->hstate.data(), b->hstate.size() * sizeof(BState), cudaMemcpyHostToDevice,
                           b->stream));
  if (b->tc) {
    // FP16 hi / lo copies of the class's rows (the datasets may have changed since the last train)
    FEM_CUDA(cudaMemsetAsync(b->terr, 0, sizeof(int), b->stream));
    k_bt_split<<<dim3(256, b->tc_nfits), 256, 0, b->stream>>>(b->fits, b->tfits, b->Xh, b->Xl);
    FEM_CUDA(cudaGetLastError());
    b->launches++;
  }
  // factorisation of the initial parameters (the fits' psum is not used)
  k_b_factor<<<b->ncomps, kBFThreads, 0, b->stream>>>(b->fits, b->state, b->comps, b->cpart, b->cfg.reg_coef, 0,
                                                      svd);
  FEM_CUDA(cudaGetLastError());
  FEM_TRY(prep_tc(b));
  k_b_sweep_end<<<1, 1024, 0, b->stream>>>(b->state, b->nfits, 0, b->cfg.max_sweeps, b->cfg.eps, b->cfg.abort_thr,
                                           svd, b->trace, b->etrace, b->cap, b->nactive);
  FEM_CUDA(cudaGetLastError());
  b->launches += 2;
  if (b->timing) FEM_CUDA(cudaEventRecord(b->ev_start, b->stream));
  int pending = 0;
  for (int it = 1; it <= b->cfg.max_sweeps; it++) {
    FEM_TRY(launch_sweep(b, it, svd, pending++));
    b->sweeps++;
    if (pending == kBatchSyncEvery || it == b->cfg.max_sweeps) {
      FEM_CUDA(cudaMemcpyAsync(b->hnactive, b->nactive, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
      FEM_CUDA(cudaStreamSynchronize(b->stream));
      if (b->timing) collect_timing(b, pending);
      pending = 0;
      if (*b->hnactive == 0) break;
    }
  }
  if (b->timing) {
    float ms = 0.f;
    FEM_CUDA(cudaEventRecord(b->ev_end, b->stream));
    FEM_CUDA(cudaEventSynchronize(b->ev_end));
    if (cudaEventElapsedTime(&ms, b->ev_start, b->ev_end) == cudaSuccess) b->t_phase[4] += ms;
  }
  FEM_CUDA(cudaMemcpyAsync(b->hstate.data(), b->state, b->hstate.size() * sizeof(BState), cudaMemcpyDeviceToHost,
                           b->stream));
  int terr = 0;
  if (b->tc) FEM_CUDA(cudaMemcpyAsync(&terr, b->terr, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  FEM_CUDA(cudaStreamSynchronize(b->stream));
  if (terr) {
    set_error("a bounded device wait timed out in the tensor-core E-step");
    return FEM_ERR_TIMEOUT;
  }
  int nfail = 0;
  for (int f = 0; f < b->nfits; f++) {
    const BState &s = b->hstate[f];
    if (status) status[f] = s.status;
    if (iter_counter) iter_counter[f] = s.iters;
    if (logl) logl[f] = s.logl;
    nfail += s.status != FEM_OK;
  }
  if (nfail) set_error("%d of %d fits stopped with an error (see the per-fit status)", nfail, b->nfits);
  return FEM_OK;
}

extern "C" int fem_em_batch_trace(fem_em_batch *b, int fit, double *logl_trace, double *e_trace, int capacity) {
  FEM_TRY(check_fit(b, fit));
  const int m = std::min(capacity, b->cap);
  FEM_CUDA(cudaSetDevice(b->cfg.device));
  if (logl_trace && m > 0)
    FEM_CUDA(cudaMemcpy(logl_trace, b->trace + (size_t)fit * b->cap, (size_t)m * sizeof(double),
                        cudaMemcpyDeviceToHost));
  if (e_trace && m > 0)
    FEM_CUDA(cudaMemcpy(e_trace, b->etrace + (size_t)fit * b->cap, (size_t)m * sizeof(double),
                        cudaMemcpyDeviceToHost));
  return FEM_OK;
}

extern "C" int fem_em_batch_fail_component(fem_em_batch *b, int fit, int *component) {
  FEM_TRY(check_fit(b, fit));
  if (!component) {
    set_error("null output");
    return FEM_ERR_BAD_ARG;
  }
  *component = b->hstate[fit].fail_comp;
  return FEM_OK;
}

extern "C" int fem_em_batch_get_tuning(fem_em_batch *b, fem_em_batch_tuning *t) {
  FEM_TRY(check_batch(b));
  if (!t) {
    set_error("null output");
    return FEM_ERR_BAD_ARG;
  }
  *t = b->tuning;
  return FEM_OK;
}

extern "C" int fem_em_batch_timing_enable(fem_em_batch *b, int on) {
  FEM_TRY(check_batch(b));
  b->timing = on != 0;
  for (double &t : b->t_phase) t = 0.0;
  for (auto &row : b->t_class)
    for (double &t : row) t = 0.0;
  b->launches = 0;
  b->sweeps = 0;
  return FEM_OK;
}

extern "C" int fem_em_batch_timing(fem_em_batch *b, double *phase_ms, int64_t *launches, int64_t *sweeps) {
  FEM_TRY(check_batch(b));
  if (phase_ms)
    for (int p = 0; p < 5; p++) phase_ms[p] = b->t_phase[p];
  if (launches) *launches = b->launches;
  if (sweeps) *sweeps = b->sweeps;
  return FEM_OK;
}

extern "C" int fem_em_batch_timing_classes(fem_em_batch *b, double *class_ms) {
  FEM_TRY(check_batch(b));
  if (!class_ms) {
    set_error("null output");
    return FEM_ERR_BAD_ARG;
  }
  for (int p = 0; p < 3; p++)
    for (int c = 0; c < kClasses; c++) class_ms[p * kClasses + c] = b->t_class[p][c];
  return FEM_OK;
}
