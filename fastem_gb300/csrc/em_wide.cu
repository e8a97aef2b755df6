// em_wide.cu -- tcgen05 split-precision EM sweep for 64 < d <= 256.
//
// Same sweep as em_tc.cu (SimpleMatrixEM::PrecomputeDensityMatrix + MStep,
// EM2/MatrixEM.cpp:275-378), organised for wide and ill-conditioned
// components (covariance condition numbers up to ~1e6), where the d <= 64
// kernels' formulation stops being accurate:
//
//  * The Mahalanobis products y = L^-1 (x - mu) cancel heavily when x is far
//    from the origin in units of the smallest eigenvalue, so x is centred per
//    component BEFORE it is rounded: a = x - m_j with m_j = fp16(mu_j) is
//    exact in FP32 (x and m_j share the FP32 grid of x), and the rest of the
//    offset, b_j = L_j^-1 (mu_j - m_j), is formed in FP64.  Rounding a to
//    FP16 hi + lo then leaves an error that depends on the data, not on mu_j,
//    and averages out over the points; rounding x - mu_j directly would leave
//    the same rounding of mu_j's low bits in every point of the component.
//  * Covariance sums accumulated in data coordinates in FP32 (TMEM) lose the
//    small eigen-directions: the rounding of the large entries is ~1e6 times
//    the small eigenvalue.  The M-step therefore accumulates in whitened
//    coordinates, where every direction has unit scale:
//        N_j M_j = sum_i r_ij y_ij y_ij^T,   N_j ybar_j = sum_i r_ij y_ij,
//        mu_j' = mu_j + L_j ybar_j,  Sigma_j' = L_j (M_j - ybar_j ybar_j^T) L_j^T,
//    which is the reference's covariance around the new means
//    (EM2/MatrixEM.cpp:319-375) in exact arithmetic.
//
// Kernels:
//  1. k_wide_prep: W_j = L_j^-1 as FP16 hi + lo, rows permuted so that each
//     64-dim input chunk's nonzero part of the triangle is a row prefix, with
//     a power-of-two scale per component (its largest entry in [2^13, 2^14):
//     no FP16 overflow whatever the covariance scale, and the rows' largest
//     entries differ by sqrt(cond), so every row stays in FP16's normal range
//     up to condition ~1e9); centres m_j, offsets b_j, log coefficients.
//  2. k_wide_estep (EM2/MatrixEM.cpp:39-51,69-81): one CTA per SM walks (tile
//     of 128 points, component j) units.  The tile's FP32 rows live in tensor
//     memory; producer warps form a = x - m_j, split it into FP16 hi / lo
//     operand tiles; the MMA warp issues a_h W_l + a_l W_h + a_h W_h for the
//     triangle (N = Dp - 16 k per 16-wide k-step) into one FP32 accumulator;
//     epilogue warps subtract b_j, square and sum, keep an online
//     log-sum-exp, finish the previous tile's posteriors (FP16 hi / lo) and
//     store y as FP16 (component-major rows of dims) for the M-step.  The
//     k-steps run from the narrowest to the widest, so the epilogue can hand
//     the accumulator back 64 columns at a time (it zeroes what it read).
//  3. k_wide_cov: z = fp16(sqrt r) * y for 64-point blocks of one component,
//     M = z z^T (two M = 128 products: dims 0..127 x 0..127 and 128..255 x
//     0..255) in FP32 TMEM windows of 16384 points, flushed to FP64; producers
//     also sum r, r y and the diagonal z_a^2 in FP32 (round to nearest).  The
//     tensor core's FP32 accumulation drops an addend's bits below the
//     accumulator's ulp (toward zero): harmless for the off-diagonal sums,
//     whose increments have either sign, but the diagonal's increments are
//     all positive and would be biased low.  The (component, block) space is
//     split evenly over the CTAs.
//  4. k_wide_gather + k_wide_gemm: FP64 finalisation per component (means,
//     weights, M - ybar ybar^T, L M L^T).
//
// Every mbarrier wait is bounded: a timeout sets the status word, the roles
// leave their loops, copies and MMAs in flight are drained and tensor memory
// is released.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "em_kernels.cuh"
#include "fem_internal.cuh"
#include "tc_ptx.cuh"

namespace fem {

using namespace tc;

constexpr int kWMax = 256;          // widest padded dimension
constexpr int kWTile = 128;         // E-step points per tile (MMA M)
constexpr int kWAS = 2;             // centred-x operand ring (64-dim chunks)
constexpr int kWWS = 2;             // W operand ring (64-dim chunks)
// W stage 0 holds at most kWS0 rows: with four chunks per unit it receives
// chunks 3 and 1 (64 and 192 rows), stage 1 chunks 2 and 0 (128 and 256);
// with three or two chunks every chunk has at most 192 rows
constexpr int kWS0 = 192;
constexpr int kWCS = 4;             // ring of per-component vectors (m, b)
constexpr uint32_t kWXCol = 256;    // TMEM column of the tile's FP32 rows
// warp 0 TMA, 1 MMA, 2..5 producers, 6..13 epilogue (two groups of 4 warps that
// read alternate 64-column quarters).  14 warps are allocated as 16, which
// leaves 128 registers per thread.
constexpr int kWEThreads = 448;
constexpr int kWEpi0 = 6;           // first epilogue warp
constexpr int kVBlk = 64;           // covariance kernel: points per block
constexpr int kVS = 5;              // covariance input ring
// blocks per FP32 accumulation window (16384 points): the window sums only the
// off-diagonal terms (increments of either sign; the diagonal is summed by the
// producers), and each flush stalls the MMAs while 393 KB of FP64 partials are
// read and written
constexpr int kVWin = 256;
constexpr int kWCThreads = 448;     // warp 0 TMA, 1 MMA, 2..9 producers (one row each), 10..13 flush
constexpr int kWCFlush0 = 10;       // first flush warp
// per (CTA, component) sums: r y (kWMax), z_a^2 (kWMax), r (64 partials)
constexpr int kSPart = 2 * kWMax + kVBlk;
constexpr int kWMaxGrid = 256;      // covariance CTAs at most (a component may meet all of them)

struct __align__(1024) WESmem {
  __half ah[kWAS][kWTile * 64];   // a = x - m, FP16 hi: rows = points, 64 dims, SW128
  __half al[kWAS][kWTile * 64];   // FP16 lo
  __half wh[(kWS0 + kWMax) * 64]; // W chunk stages: rows = permuted output dims, 64 input dims
  __half wl[(kWS0 + kWMax) * 64];
  // y of one 64-column quarter per epilogue group, rows = output dims (64),
  // 128 points each: the source of the group's TMA store into Y
  __half ys[2][64 * kWTile];
  // centre m_j and offset b_j of the units in flight, fetched by the TMA warp
  // (global loads of them would put an L2 round trip into every chunk)
  float cvm[kWCS][kWMax], cvb[kWCS][kWMax];
  uint64_t a_full[kWAS], a_empty[kWAS], w_full[kWWS], w_empty[kWWS], cv_full[kWCS], cv_empty[kWCS];
  uint64_t acc_full, acc_empty[4], mma_done;
  uint32_t tmem_base;
  float ssum[2][kWTile];          // second epilogue group's partial sums of y^2 (by unit parity)
  double red[4];
};
static_assert(sizeof(WESmem) + 1024 <= 232448, "wide E-step shared memory");

struct __align__(1024) WCSmem {
  __half y[kVS][kWMax * kVBlk];   // y block (rows = dims, 64 points, SW128); z in place
  __half rh[kVS][kVBlk], rl[kVS][kVBlk];
  __half sr[kVS][kVBlk];          // fp16(sqrt r) of the block's points
  uint64_t in_full[kVS], z_full[kVS], in_empty[kVS], acc_full, acc_empty, mma_done;
  uint32_t tmem_base;
};
static_assert(sizeof(WCSmem) + 1024 <= 232448, "wide covariance shared memory");

struct WideEmPlan {
  CUtensorMap tm_wh, tm_wl, tm_y, tm_rh, tm_rl;
  CUtensorMap tm_ys;              // Y as stored by the E-step: 128 points x 64 dims
  int Dp = 0;                     // d rounded up to a multiple of 64
  int64_t np = 0;                 // posterior / y row pitch (multiple of 64)
  int64_t nbk = 0;                // 64-point blocks
  int egrid = 0, cgrid = 0, nslot = 0;
  __half *Wh = nullptr, *Wl = nullptr;   // K x Dp x Dp, permuted rows
  float *cen = nullptr;           // K x Dp centres m = fp16(mu)
  float *wsc = nullptr;           // K component scales (powers of two)
  float *wb = nullptr;            // K x Dp offsets b = W (mu - m), permuted
  float *chi = nullptr, *clo = nullptr;  // log coefficient as float hi + lo
  double *Lw = nullptr;           // K x d x d Cholesky factors of the E-step
  __half *Rh = nullptr, *Rl = nullptr;   // K x np posteriors hi / lo
  __half *Y = nullptr;            // K x Dp x np whitened offsets, FP16
  float *lsc = nullptr;           // E-step scratch: egrid x 2 x K x 128
  double *epart = nullptr;        // per-CTA log-likelihood
  double *cpart = nullptr;        // cgrid x nslot x ncols x 128 FP64 sums of z z^T
  double *spart = nullptr;        // cgrid x nslot x kSPart
  double *Msc = nullptr, *Tsc = nullptr;  // K x d x d finalisation scratch
  int *err = nullptr;
  float *amax = nullptr;
};

__device__ __forceinline__ void w_store_post(__half *Rh, __half *Rl, size_t o, float r) {
  const __half h = __float2half_rn(r);
  Rh[o] = h;
  Rl[o] = __float2half_rn(r - __half2float(h));
}

__device__ __forceinline__ uint32_t h2_bits(__half2 v) { return *reinterpret_cast<uint32_t *>(&v); }

// FP32 -> FP16, round to nearest, values beyond the FP16 range to +-65504
__device__ __forceinline__ __half half_satfinite(float x) {
  unsigned short u;
  asm("cvt.rn.satfinite.f16.f32 %0, %1;" : "=h"(u) : "f"(x));
  return __ushort_as_half(u);
}

// ============================================================== prepare
// Row k of W_j (output dim k) goes to row p = Dp - 1 - k, scaled by 2^-e so
// that the component's largest entry lies in [2^13, 2^14) (wsc = 2^e undoes
// it on the accumulator); padded rows and columns are zero.
__global__ void __launch_bounds__(256)
k_wide_prep(const double *__restrict__ linv, const double *__restrict__ chol, const double *__restrict__ mu,
            const double *__restrict__ logc, int d, int Dp, __half *__restrict__ Wh, __half *__restrict__ Wl,
            float *__restrict__ cen, float *__restrict__ wsc, float *__restrict__ wb, float *__restrict__ chi,
            float *__restrict__ clo, double *__restrict__ Lw) {
  const int j = blockIdx.x;
  const double *Wi = linv + (size_t)j * d * d;
  const double *A = chol + (size_t)j * d * d;
  __shared__ double dm[kWMax];      // mu - m
  __shared__ double rmax[256];
  __shared__ double s_rsc;          // 2^-e
  for (int e = threadIdx.x; e < Dp; e += blockDim.x) {
    double m = 0.0, r = 0.0;
    if (e < d) {
      const double u = mu[(size_t)j * d + e];
      m = fabs(u) < 32768.0 ? (double)__half2float(__double2half(u)) : 0.0;
      r = u - m;
    }
    cen[(size_t)j * Dp + e] = (float)m;
    dm[e] = r;
  }
  double mx = 0.0;
  for (int e = threadIdx.x; e < d * d; e += blockDim.x) mx = fmax(mx, fabs(Wi[e]));
  rmax[threadIdx.x] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int t = 0; t < (int)blockDim.x; t++) m = fmax(m, rmax[t]);
    int ex = 0;
    if (m > 0.0) frexp(m, &ex);     // m = f 2^ex, f in [0.5, 1)
    const int sh = ex - 14;         // m 2^-sh in [2^13, 2^14)
    s_rsc = ldexp(1.0, -sh);
    wsc[j] = (float)ldexp(1.0, sh);
  }
  __syncthreads();
  const double rsc = s_rsc;
  for (int e = threadIdx.x; e < Dp * Dp; e += blockDim.x) {
    const int k = e / Dp, c = e - k * Dp;
    const double w = (k < d && c <= k) ? Wi[(size_t)k * d + c] * rsc : 0.0;
    const __half h = __double2half(w);
    const size_t o = ((size_t)j * Dp + (Dp - 1 - k)) * Dp + c;
    Wh[o] = h;
    Wl[o] = __double2half(w - (double)__half2float(h));
  }
  for (int k = threadIdx.x; k < Dp; k += blockDim.x) {
    double b = 0.0;
    if (k < d)
      for (int c = 0; c <= k; c++) b += Wi[(size_t)k * d + c] * dm[c];
    wb[(size_t)j * Dp + (Dp - 1 - k)] = (float)b;
  }
  for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
    const int r = e / d, c = e - r * d;
    Lw[(size_t)j * d * d + e] = c <= r ? A[e] : 0.0;
  }
  if (threadIdx.x == 0) {
    chi[j] = (float)logc[j];
    clo[j] = (float)(logc[j] - (double)(float)logc[j]);
  }
}

// ============================================================== E-step
__device__ __forceinline__ __half *w_stage(__half *w, int s) { return w + (s ? kWS0 * 64 : 0); }

__global__ void __launch_bounds__(kWEThreads, 1)
k_wide_estep(const __grid_constant__ CUtensorMap tm_wh, const __grid_constant__ CUtensorMap tm_wl,
             const __grid_constant__ CUtensorMap tm_ys, const float *__restrict__ X, const float *__restrict__ cen, const float *__restrict__ wsc,
             const float *__restrict__ wb, const float *__restrict__ chi, const float *__restrict__ clo,
             const double *__restrict__ c64, float *__restrict__ lsc, __half *__restrict__ Rh,
             __half *__restrict__ Rl, __half *__restrict__ Y, int64_t np, double *__restrict__ part, int64_t n,
             int d, int Dp, int K, int *err) {
  extern __shared__ uint8_t smem_raw[];
  WESmem &S = smem_aligned<WESmem>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nc = Dp / 64;
  const int64_t ntiles = (n + kWTile - 1) / kWTile;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kWAS; s++) mbar_init(&S.a_full[s], 4), mbar_init(&S.a_empty[s], 1);
    for (int s = 0; s < kWWS; s++) mbar_init(&S.w_full[s], 1), mbar_init(&S.w_empty[s], 1);
    // a slot is released by the 4 producer and the 8 epilogue warps
    for (int s = 0; s < kWCS; s++) mbar_init(&S.cv_full[s], 1), mbar_init(&S.cv_empty[s], 12);
    mbar_init(&S.acc_full, 1);
    for (int q = 0; q < 4; q++) mbar_init(&S.acc_empty[q], 4);
    mbar_init(&S.mma_done, 1);
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&S.tmem_base, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tmem_base;

  if (warp == 0) {
    // ------------------------------------------------ TMA: W chunks, narrowest first
    if (elect_one()) {
      tma_prefetch_desc(&tm_wh);
      tma_prefetch_desc(&tm_wl);
      uint32_t wi = 0, ci = 0;
      bool ok = true;
      for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x)
        for (int j = 0; j < K && ok; j++, ci++) {
          const int cs = ci % kWCS;
          if (!(ok = mbar_wait(&S.cv_empty[cs], ((ci / kWCS) & 1) ^ 1, err))) break;
          mbar_expect_tx(&S.cv_full[cs], (uint32_t)Dp * 8);
          bulk_load_1d(S.cvm[cs], cen + (size_t)j * Dp, (uint32_t)Dp * 4, &S.cv_full[cs]);
          bulk_load_1d(S.cvb[cs], wb + (size_t)j * Dp, (uint32_t)Dp * 4, &S.cv_full[cs]);
          for (int c = nc - 1; c >= 0; c--) {
            const int s = wi % kWWS;
            if (!(ok = mbar_wait(&S.w_empty[s], ((wi / kWWS) & 1) ^ 1, err))) break;
            const int rows = Dp - 64 * c;   // the triangle's nonzero rows of chunk c
            mbar_expect_tx(&S.w_full[s], (uint32_t)rows * 256);
            for (int rb = 0; rb < rows / 64; rb++) {
              tma_load_2d(w_stage(S.wh, s) + rb * 64 * 64, &tm_wh, &S.w_full[s], 64 * c, j * Dp + 64 * rb);
              tma_load_2d(w_stage(S.wl, s) + rb * 64 * 64, &tm_wl, &S.w_full[s], 64 * c, j * Dp + 64 * rb);
            }
            wi++;
          }
        }
      for (int s = 0; s < kWWS && wi > (uint32_t)s; s++) {
        const uint32_t u = wi - 1 - s;
        mbar_wait_drain(&S.w_full[u % kWWS], (u / kWWS) & 1);
      }
      for (int s = 0; s < kWCS && ci > (uint32_t)s; s++) {
        const uint32_t u = ci - 1 - s;
        mbar_wait_drain(&S.cv_full[u % kWCS], (u / kWCS) & 1);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (elect_one()) {
      uint32_t ai = 0, wi = 0, ui = 0;
      bool ok = true;
      for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x)
        for (int j = 0; j < K && ok; j++, ui++) {
          for (int c = nc - 1; c >= 0 && ok; c--) {
            // chunk c writes columns [0, Dp - 64c): their quarter nc - 1 - c must be
            // read and zeroed by the epilogue (arrival ui of that barrier)
            if (!(ok = mbar_wait(&S.acc_empty[nc - 1 - c], ui & 1, err))) break;
            const int sa = ai % kWAS, sw = wi % kWWS;
            if (!(ok = mbar_wait(&S.a_full[sa], (ai / kWAS) & 1, err))) break;
            if (!(ok = mbar_wait(&S.w_full[sw], (wi / kWWS) & 1, err))) break;
            tc_fence_after();
            const uint64_t dah = sdesc_sw128(smem_u32(S.ah[sa])), dal = sdesc_sw128(smem_u32(S.al[sa]));
            const uint64_t dwh = sdesc_sw128(smem_u32(w_stage(S.wh, sw)));
            const uint64_t dwl = sdesc_sw128(smem_u32(w_stage(S.wl, sw)));
#pragma unroll
            for (int t = 3; t >= 0; t--) {
              // +32 bytes per 16-element k-step inside the 128-byte swizzle row
              const uint32_t id = idesc_f16(kWTile, Dp - 16 * (4 * c + t));
              mma_f16(tbase, dah + 2 * t, dwl + 2 * t, id, 1u);
              mma_f16(tbase, dal + 2 * t, dwh + 2 * t, id, 1u);
              mma_f16(tbase, dah + 2 * t, dwh + 2 * t, id, 1u);
            }
            mma_commit(&S.a_empty[sa]);
            mma_commit(&S.w_empty[sw]);
            ai++;
            wi++;
          }
          if (!ok) break;
          mma_commit(&S.acc_full);
        }
      mma_commit(&S.mma_done);
      mbar_wait_drain(&S.mma_done, 0);
    }
  } else if (warp < kWEpi0) {
    // ------------------------------------------------ producers: a = x - m -> FP16 hi / lo
    const int quad = warp & 3, row = quad * 32 + lane;
    const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
    uint32_t ai = 0, ci = 0;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
      const int64_t pt = tile * kWTile + row;
      const bool live = pt < n;
      const float *xr = X + (live ? pt : 0) * (int64_t)d;
      // this group's part of the tile's FP32 row -> TMEM columns kWXCol ..
      for (int c = 0; c < nc; c++) {
#pragma unroll
        for (int pg = 0; pg < 2; pg++) {
          uint32_t v[32];
          const int c0 = 64 * c + 32 * pg;
          if ((d & 3) == 0) {
#pragma unroll
            for (int e = 0; e < 32; e += 4) {
              float4 x4 = make_float4(0.f, 0.f, 0.f, 0.f);
              if (live && c0 + e < d) x4 = __ldg(reinterpret_cast<const float4 *>(xr + c0 + e));
              v[e] = __float_as_uint(x4.x), v[e + 1] = __float_as_uint(x4.y);
              v[e + 2] = __float_as_uint(x4.z), v[e + 3] = __float_as_uint(x4.w);
            }
          } else {
#pragma unroll
            for (int e = 0; e < 32; e++) v[e] = __float_as_uint(live && c0 + e < d ? __ldg(xr + c0 + e) : 0.f);
          }
          tmem_st32(tbase + lane_addr + kWXCol + c0, v);
        }
      }
      tmem_wait_st();
      for (int j = 0; j < K && ok; j++, ci++) {
        const int cs = ci % kWCS;
        if (!(ok = mbar_wait_warp(&S.cv_full[cs], (ci / kWCS) & 1, err))) break;
        const float *mj = S.cvm[cs];
        for (int c = nc - 1; c >= 0; c--) {
          const int sa = ai % kWAS;
          if (!(ok = mbar_wait_warp(&S.a_empty[sa], ((ai / kWAS) & 1) ^ 1, err))) break;
          uint8_t *dh = reinterpret_cast<uint8_t *>(S.ah[sa]) + row * 128;
          uint8_t *dl = reinterpret_cast<uint8_t *>(S.al[sa]) + row * 128;
          uint32_t x[64];
          tmem_ld64(tbase + lane_addr + kWXCol + 64 * c, x);
          tmem_wait_ld();
          const float *mc = mj + 64 * c;
#pragma unroll
          for (int q = 0; q < 8; q++) {       // 16-byte chunk of the 128-byte operand row
            const float4 m0 = *reinterpret_cast<const float4 *>(mc + 8 * q);
            const float4 m1 = *reinterpret_cast<const float4 *>(mc + 8 * q + 4);
            const float a[8] = {__uint_as_float(x[8 * q]) - m0.x,     __uint_as_float(x[8 * q + 1]) - m0.y,
                                __uint_as_float(x[8 * q + 2]) - m0.z, __uint_as_float(x[8 * q + 3]) - m0.w,
                                __uint_as_float(x[8 * q + 4]) - m1.x, __uint_as_float(x[8 * q + 5]) - m1.y,
                                __uint_as_float(x[8 * q + 6]) - m1.z, __uint_as_float(x[8 * q + 7]) - m1.w};
            uint32_t hw[4], lw[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const __half2 hh = __floats2half2_rn(a[2 * u], a[2 * u + 1]);
              const float2 f = __half22float2(hh);
              hw[u] = h2_bits(hh);
              lw[u] = h2_bits(__floats2half2_rn(a[2 * u] - f.x, a[2 * u + 1] - f.y));
            }
            const int off = (q ^ (row & 7)) << 4;   // 128-byte swizzle of 16-byte chunks
            *reinterpret_cast<uint4 *>(dh + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
            *reinterpret_cast<uint4 *>(dl + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
          }
          fence_async_shared();
          __syncwarp();
          if (lane == 0) mbar_arrive(&S.a_full[sa]);
          ai++;
        }
        if (!ok) break;
        __syncwarp();
        if (lane == 0) mbar_arrive(&S.cv_empty[cs]);
      }
    }
  } else {
    // ------------------------------------------------ epilogue
    // group eg reads the 64-column quarters q with q % 2 == eg (quarters 0 and
    // 1, which the next unit's first chunks need, are handed back first); group
    // 0 also keeps the log-sum-exp and writes the posteriors
    const int quad = warp & 3, row = quad * 32 + lane, eg = (warp - kWEpi0) >> 2;
    const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
    // y leaves through the group's staging tile and one TMA store per quarter
    // (64 dims x 128 points, whole 256-byte rows): written by the threads
    // directly, y would go out as 64-byte pieces of 64 rows 2 np bytes apart,
    // and those scattered stores took half of the kernel's time
    const int gbar = 3 + eg;                      // the group's named barrier
    const bool issuer = warp == kWEpi0 + 4 * eg && lane == 0;
    __half *ys = S.ys[eg];
    // l_ij scratch of this CTA: [tile parity][component][128 points]
    float *scr = lsc + (size_t)blockIdx.x * 2 * K * kWTile + row;
    // the accumulator starts at zero and is zeroed as it is read: every MMA accumulates
    for (int q = eg; q < nc; q += 2) {
      tmem_zero32(tbase + lane_addr + 64 * q);
      tmem_zero32(tbase + lane_addr + 64 * q + 32);
    }
    tmem_wait_st();
    tc_fence_before();
    __syncwarp();
    if (lane == 0)
      for (int q = eg; q < nc; q += 2) mbar_arrive(&S.acc_empty[q]);
    double lsum = 0.0;
    bool ok = true, have_prev = false;
    int prev_par = 0;
    int64_t prev_i = -1;
    float prev_lse = 0.f;
    uint32_t ui = 0;
    int tcnt = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, tcnt++) {
      const int par = tcnt & 1;
      const int64_t pi = (tile * kWTile + row < n) ? tile * kWTile + row : -1;
      float mx = -INFINITY, se = 0.f, smax = 0.f;
      int jmax = 0;
      for (int j = 0; j < K; j++, ui++) {
        float lp = 0.f;
        if (eg == 0 && have_prev && prev_i >= 0) lp = scr[(size_t)(prev_par * K + j) * kWTile];
        const int cs = ui % kWCS;
        ok = mbar_wait_warp(&S.acc_full, ui & 1, err);
        if (ok) ok = mbar_wait_warp(&S.cv_full[cs], (ui / kWCS) & 1, err);
        // the group's warps take the same branch (its named barrier is inside)
        ok = bar_and(gbar, 128, ok);
        float s4[4] = {0.f, 0.f, 0.f, 0.f};
        if (ok) {
          tc_fence_after();
          const float *bj = S.cvb[cs];
          const float sc = wsc[j];
          for (int q = eg; q < nc; q += 2) {
            uint32_t v[64];
            tmem_ld64(tbase + lane_addr + 64 * q, v);
            tmem_wait_ld();
            tmem_zero32(tbase + lane_addr + 64 * q);
            tmem_zero32(tbase + lane_addr + 64 * q + 32);
            tmem_wait_st();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.acc_empty[q]);
            // the staging tile is free once the group's previous store has read it
            if (issuer) bulk_wait_read();
            named_bar_sync(gbar, 128);
#pragma unroll
            for (int u = 0; u < 16; u++) {
              const int p0 = 64 * q + 4 * u;
              const float4 b = *reinterpret_cast<const float4 *>(bj + p0);
              const float y[4] = {fmaf(__uint_as_float(v[4 * u]), sc, -b.x),
                                  fmaf(__uint_as_float(v[4 * u + 1]), sc, -b.y),
                                  fmaf(__uint_as_float(v[4 * u + 2]), sc, -b.z),
                                  fmaf(__uint_as_float(v[4 * u + 3]), sc, -b.w)};
#pragma unroll
              for (int e = 0; e < 4; e++) {
                s4[e] = fmaf(y[e], y[e], s4[e]);
                // output dim k = Dp - 1 - p, staging row k - (Dp - 64 - 64 q); |y|
                // beyond the FP16 range only occurs where the posterior is 0 (the
                // M-step multiplies it by sqrt r = 0)
                ys[(63 - 4 * u - e) * kWTile + row] = half_satfinite(y[e]);
              }
            }
            fence_async_shared();
            named_bar_sync(gbar, 128);
            // points past n are not written (the tensor map's extent)
            if (issuer) {
              tma_store_2d(&tm_ys, ys, (int)(tile * kWTile), j * Dp + Dp - 64 - 64 * q);
              bulk_commit();
            }
          }
          __syncwarp();
          if (lane == 0) mbar_arrive(&S.cv_empty[cs]);
        }
        float s = (s4[0] + s4[1]) + (s4[2] + s4[3]);
        if (eg == 1) S.ssum[ui & 1][row] = s;
        // both groups leave together when a wait gave up
        if (!(ok = bar_and(2, 256, ok))) break;
        if (eg == 1) continue;
        s += S.ssum[ui & 1][row];
        if (have_prev && prev_i >= 0) w_store_post(Rh, Rl, (size_t)j * np + prev_i, expf(lp - prev_lse));
        // c_j carried as float hi + lo
        const float l = (chi[j] - 0.5f * s) + clo[j];
        scr[(size_t)(par * K + j) * kWTile] = l;
        if (l > mx) {
          se = se * __expf(mx - l) + 1.f;
          mx = l;
          jmax = j;
          smax = s;
        } else if (l > -INFINITY) {
          se += __expf(l - mx);
        }
      }
      if (!ok) break;
      prev_i = pi;
      prev_lse = mx + __logf(se);
      if (pi >= 0) lsum += c64[jmax] - 0.5 * (double)smax + (double)__logf(se);
      prev_par = par;
      have_prev = true;
    }
    if (eg == 0) {
      if (ok && have_prev && prev_i >= 0)
        for (int j = 0; j < K; j++)
          w_store_post(Rh, Rl, (size_t)j * np + prev_i, expf(scr[(size_t)(prev_par * K + j) * kWTile] - prev_lse));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
      if (lane == 0) S.red[warp - kWEpi0] = lsum;
      asm volatile("bar.sync 1, 128;" ::: "memory");
      if (threadIdx.x == kWEpi0 * 32) part[blockIdx.x] = ((S.red[0] + S.red[1]) + S.red[2]) + S.red[3];
    }
    if (issuer) bulk_wait_all();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tbase, 512);
}

// ============================================================== M-step sums
// One warp's share of a window flush: the 32-column groups g = t, t + 3, ...
// of the FP32 window (TMEM lanes of the warp's quarter) added to the FP64
// partials (or stored, for a slot's first window).  The three warps of a
// lane quarter (two producer warps and one flush warp) take t = 0, 1, 2.
__device__ __forceinline__ void wide_flush_share(uint32_t taddr, double *cp, int ncols, int t, bool first) {
  for (int g = t; g < ncols / 32; g += 3) {
    const int c0 = 32 * g;
    uint32_t v[32];
    tmem_ld32(taddr + c0, v);
    tmem_wait_ld();
    if (first) {
#pragma unroll
      for (int e = 0; e < 32; e++) cp[(size_t)(c0 + e) * 128] = (double)__uint_as_float(v[e]);
    } else {
      double o[32];
#pragma unroll
      for (int e = 0; e < 32; e++) o[e] = cp[(size_t)(c0 + e) * 128];
#pragma unroll
      for (int e = 0; e < 32; e++) cp[(size_t)(c0 + e) * 128] = o[e] + (double)__uint_as_float(v[e]);
    }
  }
}

// CTA c owns blocks [c T / G, (c + 1) T / G) of the component-major
// (component, 64-point block) space, T = K nbk; slot = component - first
// component of the range.
__global__ void __launch_bounds__(kWCThreads, 1)
k_wide_cov(const __grid_constant__ CUtensorMap tm_y, const __grid_constant__ CUtensorMap tm_rh,
           const __grid_constant__ CUtensorMap tm_rl, int64_t nbk, int K, int Dp, int nslot,
           double *__restrict__ cpart, double *__restrict__ spart, int *err) {
  extern __shared__ uint8_t smem_raw[];
  WCSmem &S = smem_aligned<WCSmem>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t T = (int64_t)K * nbk;
  const int64_t f0 = (int64_t)blockIdx.x * T / gridDim.x, f1 = (int64_t)(blockIdx.x + 1) * T / gridDim.x;
  const int j0 = (int)(f0 / nbk);
  const int ncols = Dp > 128 ? 384 : 128;

  // rows Dp..255 of every stage stay zero (the copies fill rows < Dp)
  if (Dp < kWMax)
    for (int e = threadIdx.x; e < kVS * (kWMax - Dp) * 8; e += blockDim.x) {
      const int s = e / ((kWMax - Dp) * 8), r = e - s * (kWMax - Dp) * 8;
      reinterpret_cast<uint4 *>(S.y[s] + Dp * kVBlk)[r] = make_uint4(0, 0, 0, 0);
    }
  if (threadIdx.x == 0) {
    for (int s = 0; s < kVS; s++) mbar_init(&S.in_full[s], 1), mbar_init(&S.z_full[s], 8), mbar_init(&S.in_empty[s], 1);
    mbar_init(&S.acc_full, 1);
    mbar_init(&S.acc_empty, 12);   // the 8 producer and 4 flush warps
    mbar_init(&S.mma_done, 1);
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&S.tmem_base, 512);
  fence_async_shared();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tmem_base;

  if (warp == 0) {
    // ------------------------------------------------ TMA: y block + posteriors
    if (elect_one()) {
      tma_prefetch_desc(&tm_y);
      tma_prefetch_desc(&tm_rh);
      tma_prefetch_desc(&tm_rl);
      uint32_t i = 0;
      bool ok = true;
      for (int64_t f = f0; f < f1 && ok; f++, i++) {
        const int j = (int)(f / nbk);
        const int x0 = (int)((f - (int64_t)j * nbk) * kVBlk);
        const int s = i % kVS;
        if (!(ok = mbar_wait(&S.in_empty[s], ((i / kVS) & 1) ^ 1, err))) break;
        mbar_expect_tx(&S.in_full[s], (uint32_t)Dp * 128 + 2 * kVBlk * 2);
        for (int q = 0; q < Dp / 64; q++)
          tma_load_2d(S.y[s] + q * 64 * kVBlk, &tm_y, &S.in_full[s], x0, j * Dp + 64 * q);
        tma_load_2d(S.rh[s], &tm_rh, &S.in_full[s], x0, j);
        tma_load_2d(S.rl[s], &tm_rl, &S.in_full[s], x0, j);
      }
      for (int s = 0; s < kVS && i > (uint32_t)s; s++) {
        const uint32_t u = i - 1 - s;
        mbar_wait_drain(&S.in_full[u % kVS], (u / kVS) & 1);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (elect_one()) {
      uint32_t i = 0, wnd = 0;
      bool ok = true, fresh = true;
      int64_t fs = f0;
      for (int64_t f = f0; f < f1 && ok; f++, i++) {
        if (f != f0 && f % nbk == 0) fs = f;
        const int s = i % kVS;
        if (fresh) {
          if (!(ok = mbar_wait(&S.acc_empty, (wnd & 1) ^ 1, err))) break;
        }
        if (!(ok = mbar_wait(&S.z_full[s], (i / kVS) & 1, err))) break;
        tc_fence_after();
        const uint64_t dz = sdesc_sw128(smem_u32(S.y[s]));
        const uint64_t dz1 = sdesc_sw128(smem_u32(S.y[s] + 128 * kVBlk));
#pragma unroll
        for (int t = 0; t < kVBlk / 16; t++) {
          const uint32_t acc = (fresh && t == 0) ? 0u : 1u;
          mma_f16(tbase, dz + 2 * t, dz + 2 * t, idesc_f16(128, 128), acc);
          if (Dp > 128) mma_f16(tbase + 128, dz1 + 2 * t, dz + 2 * t, idesc_f16(128, 256), acc);
        }
        mma_commit(&S.in_empty[s]);
        fresh = (f == f1 - 1) || (f % nbk) == nbk - 1 || ((f - fs) % kVWin) == kVWin - 1;
        if (fresh) {
          mma_commit(&S.acc_full);
          wnd++;
        }
      }
      mma_commit(&S.mma_done);
      mbar_wait_drain(&S.mma_done, 0);
    }
  } else if (warp < kWCFlush0) {
    // ------------------------------------------------ producers: z = fp16(sqrt r) y in place
    const int p = threadIdx.x - 64;   // row p
    const int pw = warp - 2;          // producer warp 0..7
    const int quad = warp & 3;
    const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
    uint32_t i = 0, wnd = 0;
    bool ok = true, first = true;
    // block f's index within its component and position within its FP32
    // window, kept as counters (a 64-bit division per block would sit on the
    // producers' critical path)
    int64_t fb = f0 % nbk;
    int wpos = 0, slot = 0;           // slot = component of f - first component of the range
    // sum r, sum r y and sum z^2 (the diagonal: its increments are all
    // positive, which the tensor core's truncating accumulation would bias
    // low) of row p over the segment
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int64_t f = f0; f < f1 && ok; f++, i++) {
      if (f != f0 && fb == 0) first = true, wpos = 0, slot++;
      const int s = i % kVS;
      ok = mbar_wait_warp(&S.in_full[s], (i / kVS) & 1, err);
      if (ok && p < kVBlk) {
        const float r = __half2float(S.rh[s][p]) + __half2float(S.rl[s][p]);
        S.sr[s][p] = __float2half_rn(sqrtf(r));
        s0 += (double)r;
      }
      // every producer leaves together when one of them gave up (a common
      // barrier also keeps the eight warps in step: without it they drift
      // apart and the block waits for the last)
      if (!(ok = bar_and(1, 256, ok))) break;
      {
        const int rw = p;
        if (rw < Dp) {
          uint8_t *rp = reinterpret_cast<uint8_t *>(S.y[s]) + rw * 128;
          float acc = 0.f, sq = 0.f;
#pragma unroll
          for (int it = 0; it < 8; it++) {
            const int q = (it + p) & 7;       // consecutive rows start at different banks
            const int lq = q ^ (rw & 7);      // 8-point group held by physical chunk q
            uint4 v = *reinterpret_cast<uint4 *>(rp + q * 16);
            const uint4 w = *reinterpret_cast<const uint4 *>(&S.sr[s][lq * 8]);
            __half2 *vh = reinterpret_cast<__half2 *>(&v);
            const __half2 *wh = reinterpret_cast<const __half2 *>(&w);
#pragma unroll
            for (int u = 0; u < 4; u++) {
              vh[u] = __hmul2(vh[u], wh[u]);
              const float2 zf = __half22float2(vh[u]), wf = __half22float2(wh[u]);
              acc = fmaf(zf.x, wf.x, acc);
              acc = fmaf(zf.y, wf.y, acc);
              sq = fmaf(zf.x, zf.x, sq);
              sq = fmaf(zf.y, zf.y, sq);
            }
            *reinterpret_cast<uint4 *>(rp + q * 16) = v;
          }
          s1 += (double)acc;
          s2 += (double)sq;
        }
      }
      fence_async_shared();
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.z_full[s]);
      const bool send = f == f1 - 1 || fb == nbk - 1;
      if (send) {
        double *sp = spart + ((size_t)blockIdx.x * nslot + slot) * kSPart;
        sp[p] = s1;
        sp[kWMax + p] = s2;
        if (p < kVBlk) sp[2 * kWMax + p] = s0;
        s0 = 0.0, s1 = 0.0, s2 = 0.0;
      }
      // the window's flush is shared with the flush warps (the producers would
      // otherwise idle while the single accumulator is read out)
      const bool wend = send || wpos == kVWin - 1;
      wpos = wend ? 0 : wpos + 1;
      fb = fb == nbk - 1 ? 0 : fb + 1;
      if (wend) {
        // every producer reaches this point on the same block; they leave
        // together (the per-block barrier above would otherwise wait for a
        // warp that gave up here)
        ok = mbar_wait_warp(&S.acc_full, wnd & 1, err);
        if (!(ok = bar_and(1, 256, ok))) break;
        tc_fence_after();
        const int row = quad * 32 + lane;
        double *cp = cpart + ((size_t)blockIdx.x * nslot + slot) * (size_t)ncols * 128 + row;
        wide_flush_share(tbase + lane_addr, cp, ncols, pw < 4 ? 0 : 1, first);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&S.acc_empty);
        wnd++;
        first = false;
      }
    }
  } else {
    // ------------------------------------------------ flush: FP32 window -> FP64 partials
    const int quad = warp & 3, row = quad * 32 + lane;
    const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
    uint32_t wnd = 0;
    bool ok = true, first = true;
    int64_t fs = f0;
    for (int64_t f = f0; f < f1 && ok; f++) {
      if (f != f0 && f % nbk == 0) fs = f, first = true;
      const bool wend = (f == f1 - 1) || (f % nbk) == nbk - 1 || ((f - fs) % kVWin) == kVWin - 1;
      if (!wend) continue;
      if (!(ok = mbar_wait_warp(&S.acc_full, wnd & 1, err))) break;
      tc_fence_after();
      double *cp = cpart + ((size_t)blockIdx.x * nslot + ((int)(f / nbk) - j0)) * (size_t)ncols * 128 + row;
      wide_flush_share(tbase + lane_addr, cp, ncols, 2, first);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.acc_empty);
      wnd++;
      first = false;
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tbase, 512);
}

// ============================================================== finalise
// Per component: gathers the sums of the CTAs whose ranges meet it, then
// N_j, ybar, M = sum z z^T / N_j - ybar ybar^T (Msc, full symmetric d x d),
// mu' = mu + L ybar, pi = N_j / n.
__global__ void __launch_bounds__(256)
k_wide_gather(const double *__restrict__ cpart, const double *__restrict__ spart, int cg, int nslot,
              int64_t nbk, int K, int d, int Dp, int64_t n, const double *__restrict__ Lw,
              double *__restrict__ mu, double *__restrict__ pi, double *__restrict__ psum,
              double *__restrict__ Msc) {
  const int j = blockIdx.x;
  const int ncols = Dp > 128 ? 384 : 128;
  const int64_t T = (int64_t)K * nbk;
  __shared__ int s_cta[kWMaxGrid], s_slot[kWMaxGrid];
  __shared__ int s_cnt;
  __shared__ double ybar[kWMax], red[256];
  if (threadIdx.x == 0) {
    int c = 0;
    for (int g = 0; g < cg; g++) {
      const int64_t a = (int64_t)g * T / cg, b = (int64_t)(g + 1) * T / cg;
      if (a < (int64_t)(j + 1) * nbk && b > (int64_t)j * nbk && b > a) {
        s_cta[c] = g;
        s_slot[c] = j - (int)(a / nbk);
        c++;
      }
    }
    s_cnt = c;
  }
  __syncthreads();
  const int cnt = s_cnt;
  // N_j
  double r = 0.0;
  for (int e = threadIdx.x; e < cnt * kVBlk; e += blockDim.x) {
    const int u = e / kVBlk, t = e - u * kVBlk;
    r += spart[((size_t)s_cta[u] * nslot + s_slot[u]) * kSPart + 2 * kWMax + t];
  }
  red[threadIdx.x] = r;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  const double Nj = red[0];
  for (int a = threadIdx.x; a < Dp; a += blockDim.x) {
    double v = 0.0;
    for (int u = 0; u < cnt; u++) v += spart[((size_t)s_cta[u] * nslot + s_slot[u]) * kSPart + a];
    ybar[a] = v / Nj;
  }
  __syncthreads();
  // M (lower triangle from the two products, mirrored)
  double *M = Msc + (size_t)j * d * d;
  for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
    const int a = e / d, b = e - a * d;
    if (b > a) continue;
    double v = 0.0;
    for (int u = 0; u < cnt; u++) {
      if (a == b) {
        v += spart[((size_t)s_cta[u] * nslot + s_slot[u]) * kSPart + kWMax + a];
      } else {
        const double *cp = cpart + ((size_t)s_cta[u] * nslot + s_slot[u]) * (size_t)ncols * 128;
        v += (a < 128) ? cp[(size_t)b * 128 + a] : cp[(size_t)(128 + b) * 128 + (a - 128)];
      }
    }
    const double m = v / Nj - ybar[a] * ybar[b];
    M[(size_t)a * d + b] = m;
    M[(size_t)b * d + a] = m;
  }
  // mu' = mu + L ybar, weights
  const double *L = Lw + (size_t)j * d * d;
  for (int a = threadIdx.x; a < d; a += blockDim.x) {
    double v = 0.0;
    for (int b = 0; b <= a; b++) v += L[(size_t)a * d + b] * ybar[b];
    mu[(size_t)j * d + a] += v;
  }
  if (threadIdx.x == 0) {
    psum[j] = Nj;
    pi[j] = Nj / (double)n;
  }
}

// C = A B over 64 x 64 output tiles (FP64): mode 0, C = L M (L lower: inner
// blocks kk <= I); mode 1, C = T L^T for lower tiles I >= J (inner blocks
// kk <= J), mirrored to the upper triangle.  grid = (tiles, tiles, K).
__global__ void __launch_bounds__(256)
k_wide_gemm(const double *__restrict__ A, const double *__restrict__ B, double *__restrict__ C, int d, int mode) {
  const int I = blockIdx.y, J = blockIdx.x, j = blockIdx.z;
  if (mode == 1 && J > I) return;
  const size_t off = (size_t)j * d * d;
  A += off, B += off, C += off;
  __shared__ double As[64][17], Bs[16][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4] = {};
  const int kend = 64 * ((mode == 0 ? I : J) + 1);
  for (int k0 = 0; k0 < kend && k0 < d; k0 += 16) {
    for (int e = threadIdx.x; e < 64 * 16; e += 256) {
      const int r = e >> 4, c = e & 15;
      const int gr = 64 * I + r, gk = k0 + c;
      As[r][c] = (gr < d && gk < d) ? A[(size_t)gr * d + gk] : 0.0;
      // mode 0: B = M (row-major); mode 1: B = L^T, B[k][col] = L[col][k]
      const int bk = k0 + (e >> 6), bc = 64 * J + (e & 63);
      double bv = 0.0;
      if (bk < d && bc < d) bv = (mode == 0) ? B[(size_t)bk * d + bc] : B[(size_t)bc * d + bk];
      Bs[e >> 6][e & 63] = bv;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; kk++) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; u++) a[u] = As[ty + 16 * u][kk], b[u] = Bs[kk][tx + 16 * u];
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; u++)
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const int r = 64 * I + ty + 16 * u, c = 64 * J + tx + 16 * v;
      if (r >= d || c >= d) continue;
      if (mode == 0) {
        C[(size_t)r * d + c] = acc[u][v];
      } else if (c <= r) {
        C[(size_t)r * d + c] = acc[u][v];
        C[(size_t)c * d + r] = acc[u][v];
      }
    }
}

__global__ void k_wide_amax(const float *__restrict__ X, int64_t m, float *__restrict__ amax) {
  float v = 0.f;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x)
    v = fmaxf(v, fabsf(X[e]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int *>(amax), __float_as_int(v));
}

__global__ void k_wide_reduce(const double *__restrict__ part, int np, DevStatus *st, const int *__restrict__ err) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < np; b++) s += part[b];
    st->logl = s;
    if (*err) st->timeout = 1;
  }
}

__global__ void k_wide_flag(DevStatus *st, const int *__restrict__ err) {
  if (threadIdx.x == 0 && *err) st->timeout = 1;
}

__global__ void k_wide_post_rows(const __half *__restrict__ Rh, const __half *__restrict__ Rl, int64_t np, int K,
                                 int64_t r0, int64_t rows, double *__restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * K) return;
  const int64_t i = e / K;
  const int j = (int)(e - i * K);
  const size_t o = (size_t)j * np + r0 + i;
  out[e] = (double)__half2float(Rh[o]) + (double)__half2float(Rl[o]);
}

__global__ void k_wide_classes(const __half *__restrict__ Rh, const __half *__restrict__ Rl, int64_t np, int64_t n,
                               int K, int32_t *__restrict__ cls) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float best = -1.f;
  int bj = -1;
  for (int j = 0; j < K; j++) {
    const float v = __half2float(Rh[(size_t)j * np + i]) + __half2float(Rl[(size_t)j * np + i]);
    if (v > best) {
      best = v;
      bj = j;
    }
  }
  cls[i] = bj;
}

// ============================================================== host side
static size_t wesmem_bytes() { return sizeof(WESmem) + 1024; }
static size_t wcsmem_bytes() { return sizeof(WCSmem) + 1024; }

bool em_wide_supported(int d, int k) { return d > 64 && d <= kWMax && k >= 1; }

int em_wide_create(fem_em *h) {
  WideEmPlan *p = new WideEmPlan();
  h->wide = p;
  const int K = h->k, d = h->d;
  const int64_t n = h->n;
  const int Dp = (d + 63) / 64 * 64;
  p->Dp = Dp;
  p->np = (n + 63) / 64 * 64;
  p->nbk = (n + kVBlk - 1) / kVBlk;
  const int sms = sm_count();
  const int64_t ntiles = (n + kWTile - 1) / kWTile;
  p->egrid = (int)std::min<int64_t>(sms, ntiles);
  p->cgrid = (int)std::min<int64_t>(std::min(sms, kWMaxGrid), (int64_t)K * p->nbk);
  const int64_t T = (int64_t)K * p->nbk;
  const int64_t span = (T + p->cgrid - 1) / p->cgrid;   // blocks per CTA at most
  p->nslot = (int)((span + p->nbk - 1) / p->nbk) + 1;
  const size_t kdp = (size_t)K * Dp;
  FEM_TRY(dalloc(&p->Wh, kdp * Dp));
  FEM_TRY(dalloc(&p->Wl, kdp * Dp));
  FEM_TRY(dalloc(&p->cen, kdp));
  FEM_TRY(dalloc(&p->wsc, (size_t)K));
  FEM_TRY(dalloc(&p->wb, kdp));
  FEM_TRY(dalloc(&p->chi, K));
  FEM_TRY(dalloc(&p->clo, K));
  FEM_TRY(dalloc(&p->Lw, (size_t)K * d * d));
  FEM_TRY(dalloc(&p->Msc, (size_t)K * d * d));
  FEM_TRY(dalloc(&p->Tsc, (size_t)K * d * d));
  FEM_TRY(dalloc(&p->Rh, (size_t)K * p->np));
  FEM_TRY(dalloc(&p->Rl, (size_t)K * p->np));
  if (dalloc(&p->Y, kdp * p->np) != FEM_OK) {
    set_error("mixed precision at d=%d keeps the whitened offsets of every point and component: "
              "%.1f GB of device memory could not be allocated", d, (double)kdp * p->np * 2 / 1e9);
    return FEM_ERR_CUDA;
  }
  FEM_TRY(dalloc(&p->lsc, (size_t)p->egrid * 2 * K * kWTile));
  FEM_TRY(dalloc(&p->epart, p->egrid));
  const int ncols = Dp > 128 ? 384 : 128;
  FEM_TRY(dalloc(&p->cpart, (size_t)p->cgrid * p->nslot * ncols * 128));
  FEM_TRY(dalloc(&p->spart, (size_t)p->cgrid * p->nslot * kSPart));
  FEM_TRY(dalloc(&p->err, 1));
  FEM_CUDA(cudaMemset(p->err, 0, sizeof(int)));
  FEM_TRY(dalloc(&p->amax, 1));
  FEM_TRY(encode_tmap_2d(&p->tm_wh, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->Wh, (uint64_t)Dp, (uint64_t)K * Dp, 64,
                         64, CU_TENSOR_MAP_SWIZZLE_128B, (uint64_t)Dp * 2));
  FEM_TRY(encode_tmap_2d(&p->tm_wl, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->Wl, (uint64_t)Dp, (uint64_t)K * Dp, 64,
                         64, CU_TENSOR_MAP_SWIZZLE_128B, (uint64_t)Dp * 2));
  // points past n read as zero (posterior 0, y 0)
  FEM_TRY(encode_tmap_2d(&p->tm_y, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->Y, (uint64_t)n, (uint64_t)K * Dp, kVBlk,
                         64, CU_TENSOR_MAP_SWIZZLE_128B, (uint64_t)p->np * 2));
  FEM_TRY(encode_tmap_2d(&p->tm_ys, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->Y, (uint64_t)n, (uint64_t)K * Dp, kWTile,
                         64, CU_TENSOR_MAP_SWIZZLE_NONE, (uint64_t)p->np * 2));
  FEM_TRY(encode_tmap_2d(&p->tm_rh, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->Rh, (uint64_t)n, (uint64_t)K, kVBlk, 1,
                         CU_TENSOR_MAP_SWIZZLE_NONE, (uint64_t)p->np * 2));
  FEM_TRY(encode_tmap_2d(&p->tm_rl, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->Rl, (uint64_t)n, (uint64_t)K, kVBlk, 1,
                         CU_TENSOR_MAP_SWIZZLE_NONE, (uint64_t)p->np * 2));
  FEM_CUDA(cudaFuncSetAttribute(k_wide_estep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wesmem_bytes()));
  FEM_CUDA(cudaFuncSetAttribute(k_wide_cov, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wcsmem_bytes()));
  return FEM_OK;
}

void em_wide_destroy(fem_em *h) {
  WideEmPlan *p = h->wide;
  if (!p) return;
  dfree(p->Wh);
  dfree(p->Wl);
  dfree(p->cen);
  dfree(p->wsc);
  dfree(p->wb);
  dfree(p->chi);
  dfree(p->clo);
  dfree(p->Lw);
  dfree(p->Msc);
  dfree(p->Tsc);
  dfree(p->Rh);
  dfree(p->Rl);
  dfree(p->Y);
  dfree(p->lsc);
  dfree(p->epart);
  dfree(p->cpart);
  dfree(p->spart);
  dfree(p->err);
  dfree(p->amax);
  delete p;
  h->wide = nullptr;
}

int em_wide_upload(fem_em *h) {
  WideEmPlan *p = h->wide;
  FEM_CUDA(cudaMemsetAsync(p->amax, 0, sizeof(float), h->stream));
  const int64_t m = h->n * h->d;
  const int blocks = (int)std::min<int64_t>(4 * sm_count(), (m + 255) / 256);
  k_wide_amax<<<blocks, 256, 0, h->stream>>>(h->X, m, p->amax);
  float a = 0.f;
  cudaMemcpyAsync(&a, p->amax, sizeof(float), cudaMemcpyDeviceToHost, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    set_error("dataset range check failed: %s", cudaGetErrorString(e));
    return FEM_ERR_CUDA;
  }
  h->launches += 1;
  if (!(a < 32768.f)) {
    set_error("mixed precision needs |x| < 32768 (FP16 operands); max |x| = %g", a);
    return FEM_ERR_UNSUPPORTED;
  }
  return FEM_OK;
}

int em_wide_prepare(fem_em *h) {
  WideEmPlan *p = h->wide;
  k_wide_prep<<<h->k, 256, 0, h->stream>>>(h->linv, h->work, h->mu, h->logc, h->d, p->Dp, p->Wh, p->Wl, p->cen,
                                           p->wsc, p->wb, p->chi, p->clo, p->Lw);
  FEM_CUDA(cudaGetLastError());
  h->launches += 1;
  return FEM_OK;
}

int em_wide_estep(fem_em *h) {
  WideEmPlan *p = h->wide;
  k_wide_estep<<<p->egrid, kWEThreads, wesmem_bytes(), h->stream>>>(
      p->tm_wh, p->tm_wl, p->tm_ys, h->X, p->cen, p->wsc, p->wb, p->chi, p->clo, h->logc, p->lsc, p->Rh, p->Rl, p->Y, p->np,
      p->epart, h->n, h->d, p->Dp, h->k, p->err);
  FEM_CUDA(cudaGetLastError());
  k_wide_reduce<<<1, 32, 0, h->stream>>>(p->epart, p->egrid, h->dstat, p->err);
  FEM_CUDA(cudaGetLastError());
  h->launches += 2;
  return FEM_OK;
}

int em_wide_mstep(fem_em *h) {
  WideEmPlan *p = h->wide;
  const int K = h->k, d = h->d;
  timing_begin(h, 8);
  k_wide_cov<<<p->cgrid, kWCThreads, wcsmem_bytes(), h->stream>>>(p->tm_y, p->tm_rh, p->tm_rl, p->nbk, K, p->Dp,
                                                                  p->nslot, p->cpart, p->spart, p->err);
  FEM_CUDA(cudaGetLastError());
  timing_begin(h, 9);
  k_wide_gather<<<K, 256, 0, h->stream>>>(p->cpart, p->spart, p->cgrid, p->nslot, p->nbk, K, d, p->Dp, h->n, p->Lw,
                                          h->mu, h->pi, h->psum, p->Msc);
  FEM_CUDA(cudaGetLastError());
  const int tl = (d + 63) / 64;
  k_wide_gemm<<<dim3(tl, tl, K), 256, 0, h->stream>>>(p->Lw, p->Msc, p->Tsc, d, 0);
  FEM_CUDA(cudaGetLastError());
  k_wide_gemm<<<dim3(tl, tl, K), 256, 0, h->stream>>>(p->Tsc, p->Lw, h->sigma, d, 1);
  FEM_CUDA(cudaGetLastError());
  k_wide_flag<<<1, 32, 0, h->stream>>>(h->dstat, p->err);
  FEM_CUDA(cudaGetLastError());
  h->launches += 5;
  return FEM_OK;
}

int em_wide_reset_err(fem_em *h) {
  FEM_CUDA(cudaMemsetAsync(h->wide->err, 0, sizeof(int), h->stream));
  return FEM_OK;
}

int em_wide_post_rows(fem_em *h, int64_t r0, int64_t rows, double *dout) {
  WideEmPlan *p = h->wide;
  const int64_t tot = rows * h->k;
  k_wide_post_rows<<<(unsigned)((tot + 255) / 256), 256, 0, h->stream>>>(p->Rh, p->Rl, p->np, h->k, r0, rows, dout);
  FEM_CUDA(cudaGetLastError());
  return FEM_OK;
}

void em_wide_posteriors(fem_em *h, const __half **rh, const __half **rl, int64_t *pitch) {
  *rh = h->wide->Rh;
  *rl = h->wide->Rl;
  *pitch = h->wide->np;
}

int em_wide_classes(fem_em *h, int32_t *dcls) {
  WideEmPlan *p = h->wide;
  k_wide_classes<<<(unsigned)((h->n + 255) / 256), 256, 0, h->stream>>>(p->Rh, p->Rl, p->np, h->n, h->k, dcls);
  FEM_CUDA(cudaGetLastError());
  return FEM_OK;
}

}  // namespace fem
