// em_tc.cu -- tcgen05 mixed-precision EM sweep for sm_103a (d = 64).
//
// One sweep = SimpleMatrixEM::PrecomputeDensityMatrix + MStep
// (EM2/MatrixEM.cpp:275-378) as three tensor-core kernels and two FP64
// finalisers:
//
//  1. E-step (MatrixEMBase::BlockDensities + PostProcessDensityMatrix,
//     EM2/MatrixEM.cpp:39-51,69-81): ONE GEMM of the points against the
//     stacked inverse Cholesky factors of all components,
//       Y = X W^T,  W = [L_1^-1; ...; L_K^-1],  y_jk = (L_j^-1 x)_k,
//     in FP16 x 3 (x = xh + xl, W = Wh + Wl: Xh Wh^T + Xh Wl^T + Xl Wh^T)
//     with FP32 accumulation in TMEM.  A CTA works on a pair of 128-point
//     tiles so every W group fetched from L2 feeds two M=128 MMAs.  The
//     epilogue subtracts b_j = L_j^-1 mu_j (kept in shared memory), squares
//     and sums each component's 64 columns, adds the log coefficient (float
//     hi + lo) and keeps an online log-sum-exp per point; the posteriors
//     r_ij = exp(l_ij - LSE_i) of the previous pair are finished while the
//     current pair's groups drain, and stored as FP16 hi/lo pairs
//     (component-major).  The per-point log-likelihood is summed in FP64 with
//     the FP64 log coefficient of the winning component.
//     Within a group of 2 components the 128 accumulator columns are ordered
//     by 16-wide k-block, highest first, so K-step kb only needs the first
//     128-32kb columns (L^-1 is lower triangular): 37.5% of the MMA work is
//     skipped.
//  2. Means (doMStep means part, EM2/MatrixEM.cpp:319-343): S2 = R^T X and
//     S1 = R^T 1 as one GEMM per 64-point block, A = [Rh | Rl] (components
//     x points), B = [Xh^T; 1] / [Xl^T; 0] (80 rows x points); FP32 in TMEM,
//     flushed to FP64 every 4096 points.
//  3. Covariances (ComputeWeightedTempDataset + BlockCovariances,
//     EM2/MatrixEM.cpp:53-67,90-99) around the NEW means: producer warps
//     form z = sqrt(r) (x - mu_j) in FP32, store fp16(z) as the operand of
//     an M=128 (two components) x N=128 x K=16 MMA whose diagonal blocks are
//     Z_j^T Z_j, and accumulate the exact diagonal sum z^2 in FP32 -> FP64
//     (FP16 rounding would bias the diagonal upward by E[delta^2]).
//
// Every mbarrier wait is bounded; a timeout sets a status word, the roles
// leave their loops, in-flight copies and MMAs are drained and TMEM is
// released.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <vector>

#include "em_kernels.cuh"
#include "fem_internal.cuh"
#include "tc_ptx.cuh"

namespace fem {

using namespace tc;

// ------------------------------------------------------------ constants
constexpr int kD = 64;                   // dimension handled by the tensor-core path
constexpr int kTileM = 128;              // E-step points per tile (two tiles per CTA step)
constexpr int kGroupN = 128;             // E-step accumulator columns per component group
constexpr int kCompPerGroup = kGroupN / kD;
constexpr int kWStages = 4;
constexpr uint32_t kXBytes = kTileM * kD * 2;    // one FP16 X tile (16 KB)
constexpr uint32_t kWBytes = kGroupN * kD * 2;   // one FP16 W group (16 KB)
constexpr int kEThreads = 320;  // warp 0 TMA, 1 MMA, 2..9 epilogue
constexpr int kBlk = 64;                 // M-step points per block (one 128-byte swizzle row)
constexpr int kFlushBlocks = 64;         // FP32 TMEM window: 64 blocks = 4096 points
constexpr int kMaxK = 128;               // components handled by one means M-tile
constexpr int kMStages = 3;              // means input ring
constexpr int kCIn = 6;                  // covariance input ring

struct __align__(1024) ESmem {
  __half xh[2][kTileM * kD];   // the two tiles of the current pair
  __half xl[2][kTileM * kD];
  __half wh[kWStages][kGroupN * kD];
  __half wl[kWStages][kGroupN * kD];
  float bias[kMaxK * kD];      // b = L^-1 mu, permuted like the accumulator columns
  float chi[kMaxK], clo[kMaxK];
  uint64_t x_full, x_empty;
  uint64_t w_full[kWStages], w_empty[kWStages];
  uint64_t acc_full[2][2], acc_empty[2][2];   // [TMEM buffer][tile of the pair]
  uint64_t mma_done;
  uint32_t tmem_base;
  double red[8];
};

// means kernel: A = Rh/Rl (128 comps x 64 points), B = [X^T; 1] (80 x 64)
constexpr int kMeanN = 80;
struct __align__(1024) MSmem {
  __half rh[kMStages][kMaxK * kBlk];
  __half rl[kMStages][kMaxK * kBlk];
  __half bh[kMStages][kMeanN * kBlk];   // rows 0..63 X_h^T, row 64 ones, rows 65..79 zero
  __half bl[kMStages][kMeanN * kBlk];   // rows 0..63 X_l^T, rows 64..79 zero
  uint64_t in_full[kMStages], in_empty[kMStages], acc_full[2], acc_empty[2], mma_done;
  uint32_t tmem_base;
};

// covariance kernel: 4 components per CTA (2 pairs), 64-point blocks
constexpr int kZStages = 3;              // operand (z) ring
constexpr int kCProd = 16;               // producer warps: 2 groups x 8 point chunks
struct __align__(1024) CSmem {
  __half z[kZStages][2][128 * kBlk];  // [stage][pair] 128 rows (comp q dims) x 64 points, SW128
  float xs[kCIn][kBlk * kD];     // X tile (points x dims)
  __half rh[kCIn][4 * kBlk];
  __half rl[kCIn][4 * kBlk];
  float sr[kCProd][4 * 8];       // per producer warp: sqrt(r) of its 8 points x 4 components
  double dred[8][4][kD];         // exact-diagonal partials of the 8 point chunks
  uint64_t in_full[kCIn], in_empty[kCIn], z_full[kZStages], z_empty[kZStages], acc_full[2], acc_empty[2],
      mma_done;
  uint32_t tmem_base;
};
constexpr int kCThreads = (2 + kCProd + 4) * 32;   // warp 0 TMA, 1 MMA, 2..17 producers, 18..21 flush
static_assert(sizeof(CSmem) + 1024 <= 232448, "covariance kernel shared memory");

// covariance kernel, z x^T form: 4 components per CTA (2 pairs), 64-point blocks
#ifndef FEM_COV_GROUPS
#define FEM_COV_GROUPS 4
#endif
#ifndef FEM_COV_SPLIT
#define FEM_COV_SPLIT 2
#endif
#ifndef FEM_COV_STAGGER
#define FEM_COV_STAGGER 0
#endif
constexpr int kZIn = 6;                  // input ring (blocks)
constexpr int kZA = 3;                   // TMEM A ring (blocks of 64 points, both pairs)
constexpr int kZSets = FEM_COV_GROUPS;   // producer groups of 4 warps (one per TMEM lane quarter)
constexpr int kZSplit = FEM_COV_SPLIT;   // groups sharing a block (each takes kBlk / 16 / kZSplit K steps)
constexpr int kZStagger = FEM_COV_STAGGER;
constexpr int kZN = 80;                  // accumulator columns per pair: 64 (x) + 16 (column 64 = sum z)
constexpr uint32_t kZDCol = kZN;         // accumulator column pitch (pairs, buffers)
constexpr uint32_t kZACol = 4 * kZN;     // first column of the A ring
constexpr uint32_t kZAStage = 2 * (kBlk / 2);   // A columns per block: 2 pairs x 32 (64 FP16 points)
constexpr int kZThreads = (2 + 4 * kZSets + 4) * 32;   // TMA, MMA, producers, flush
constexpr int kZCols = kD + 1;           // flushed columns per pair row: 64 sums z x_b, then sum z
struct __align__(1024) ZSmem {
  __half bh[kZIn][kZN * kBlk];   // rows 0..63 X_h^T (TMA), row 64 ones, rows 65..79 zero (SW128)
  __half bl[kZIn][kD * kBlk];    // X_l^T (TMA, SW128)
  __half rh[kZIn][4 * kBlk];     // posteriors (hi part) of the CTA's 4 components
  uint64_t in_full[kZIn], in_empty[kZIn], a_full[kZA], a_empty[kZA], acc_full[2], acc_empty[2], mma_done;
  uint32_t tmem_base;
};
static_assert(sizeof(ZSmem) + 1024 <= 232448, "covariance kernel shared memory");
static_assert(kZSets % kZSplit == 0 && (kBlk / 16) % kZSplit == 0, "covariance producer split");
static_assert(kZACol + kZA * kZAStage <= 512 && 3 * kZDCol + kZN <= kZACol, "covariance kernel TMEM columns");

struct TcEmPlan {
  CUtensorMap tm_xh, tm_xl, tm_wh, tm_wl;      // E-step
  CUtensorMap tm_rh, tm_rl, tm_xht, tm_xlt;    // means
  CUtensorMap tm_x32, tm_rh4, tm_rl4;          // covariances
  __half *Wh = nullptr, *Wl = nullptr;  // (K*d) x d, permuted rows
  float *bias = nullptr;                // K*d, permuted
  float *clo = nullptr;                 // log coefficient - float(log coefficient)
  __half *Rh = nullptr, *Rl = nullptr;  // K x np posteriors hi / lo
  __half *XhT = nullptr, *XlT = nullptr;  // d x np
  int64_t np = 0;                       // padded row pitch (multiple of 64)
  float *lsc = nullptr;                 // E-step scratch: egrid x 2 x K x 256
  double *epart = nullptr;              // per-CTA log-likelihood
  double *mpart = nullptr;              // means partials: mgrid x 80 columns x 128 components
  double *cpart = nullptr;              // covariance partials: cgrid x 2 pairs x 64 columns x 128 rows
  double *dpart = nullptr;              // exact diagonals: cgrid x 4 x 64
  float *muf = nullptr;                 // new means (float) for the covariance producers
  float *chi = nullptr;                 // float(log coefficient); -inf for padding components
  float *X64 = nullptr;                 // n x 64 zero-padded FP32 rows when d < 64
  int *err = nullptr;                   // device status of the bounded waits
  float *amax = nullptr;                // upload: largest |x| (FP16 range check)
  int *roles = nullptr;                 // bounded-wait expiry self-test: which waits gave up
  int egrid = 0, mgrid = 0, cgx = 0, cgy = 0;
  int kp = 0, d = 0;                    // components padded to a multiple of 4; true dimension
};

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void store_post(__half *Rh, __half *Rl, size_t o, float r) {
  const __half h = __float2half_rn(r);
  Rh[o] = h;
  Rl[o] = __float2half_rn(r - __half2float(h));
}

// ============================================================== E-step
__global__ void __launch_bounds__(kEThreads, 1)
k_estep_tc(const __grid_constant__ CUtensorMap tm_xh, const __grid_constant__ CUtensorMap tm_xl,
           const __grid_constant__ CUtensorMap tm_wh, const __grid_constant__ CUtensorMap tm_wl,
           const float *__restrict__ bias, const float *__restrict__ chi, const float *__restrict__ clo,
           const double *__restrict__ c64, float *__restrict__ lsc, __half *__restrict__ Rh,
           __half *__restrict__ Rl, int64_t np, double *__restrict__ part, int64_t n, int K, int *err) {
  extern __shared__ uint8_t smem_raw[];
  ESmem &S = smem_aligned<ESmem>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int G = K / kCompPerGroup;
  const int64_t ntiles = (n + kTileM - 1) / kTileM;
  const int64_t npairs = (ntiles + 1) / 2;

  for (int e = threadIdx.x; e < K * kD; e += blockDim.x) S.bias[e] = bias[e];
  for (int j = threadIdx.x; j < K; j += blockDim.x) S.chi[j] = chi[j], S.clo[j] = clo[j];
  if (threadIdx.x == 0) {
    mbar_init(&S.x_full, 1), mbar_init(&S.x_empty, 1);
    for (int s = 0; s < kWStages; s++) mbar_init(&S.w_full[s], 1), mbar_init(&S.w_empty[s], 1);
    for (int s = 0; s < 2; s++)
      for (int t = 0; t < 2; t++) mbar_init(&S.acc_full[s][t], 1), mbar_init(&S.acc_empty[s][t], 4);
    mbar_init(&S.mma_done, 1);
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&S.tmem_base, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tmem_base;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (elect_one()) {
      tma_prefetch_desc(&tm_xh);
      tma_prefetch_desc(&tm_xl);
      tma_prefetch_desc(&tm_wh);
      tma_prefetch_desc(&tm_wl);
      uint32_t xi = 0, wi = 0;
      bool ok = true;
      for (int64_t pr = blockIdx.x; pr < npairs && ok; pr += gridDim.x) {
        if (!(ok = mbar_wait_lazy(&S.x_empty, (xi & 1) ^ 1, err, 128))) break;
        const bool has1 = 2 * pr + 1 < ntiles;
        mbar_expect_tx(&S.x_full, (has1 ? 4 : 2) * kXBytes);
        tma_load_2d(S.xh[0], &tm_xh, &S.x_full, 0, (int)(2 * pr * kTileM));
        tma_load_2d(S.xl[0], &tm_xl, &S.x_full, 0, (int)(2 * pr * kTileM));
        if (has1) {
          tma_load_2d(S.xh[1], &tm_xh, &S.x_full, 0, (int)((2 * pr + 1) * kTileM));
          tma_load_2d(S.xl[1], &tm_xl, &S.x_full, 0, (int)((2 * pr + 1) * kTileM));
        }
        xi++;
        for (int g = 0; g < G; g++) {
          const int ws = wi % kWStages;
          if (!(ok = mbar_wait_lazy(&S.w_empty[ws], ((wi / kWStages) & 1) ^ 1, err, 128))) break;
          mbar_expect_tx(&S.w_full[ws], 2 * kWBytes);
          tma_load_2d(S.wh[ws], &tm_wh, &S.w_full[ws], 0, g * kGroupN);
          tma_load_2d(S.wl[ws], &tm_wl, &S.w_full[ws], 0, g * kGroupN);
          wi++;
        }
      }
      // drain: the last loads must land before the CTA may exit
      if (xi > 0) mbar_wait_drain(&S.x_full, (xi - 1) & 1);
      for (int s = 0; s < kWStages && wi > (uint32_t)s; s++) {
        const uint32_t u = wi - 1 - s;
        mbar_wait_drain(&S.w_full[u % kWStages], (u / kWStages) & 1);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (elect_one()) {
      uint32_t xi = 0, wi = 0, ai = 0;
      bool ok = true;
      for (int64_t pr = blockIdx.x; pr < npairs && ok; pr += gridDim.x) {
        if (!(ok = mbar_wait(&S.x_full, xi & 1, err))) break;
        tc_fence_after();
        const int nt = (2 * pr + 1 < ntiles) ? 2 : 1;
        uint64_t dxh[2], dxl[2];
        for (int t = 0; t < 2; t++) {
          dxh[t] = sdesc_sw128(smem_u32(S.xh[t]));
          dxl[t] = sdesc_sw128(smem_u32(S.xl[t]));
        }
        for (int g = 0; g < G; g++) {
          const int ws = wi % kWStages, ab = ai & 1;
          if (!(ok = mbar_wait(&S.w_full[ws], (wi / kWStages) & 1, err))) break;
          const uint64_t dwh = sdesc_sw128(smem_u32(S.wh[ws]));
          const uint64_t dwl = sdesc_sw128(smem_u32(S.wl[ws]));
          // each tile has its own accumulator barriers, so its epilogue warps
          // start as soon as its own products are done; a pair with one tile
          // still completes the second tile's phases (no products)
          for (int t = 0; t < 2; t++) {
            if (!(ok = mbar_wait(&S.acc_empty[ab][t], ((ai >> 1) & 1) ^ 1, err))) break;
            tc_fence_after();
            if (t < nt) {
              const uint32_t dt = tbase + (2 * ab + t) * kGroupN;
              // the small cross products Xh Wl and Xl Wh first, Xh Wh last: the
              // accumulator is rounded after every MMA, and it only grows to
              // |W x| during the final four steps
#pragma unroll
              for (int p = 0; p < 3; p++) {
                const uint64_t da = (p == 1) ? dxl[t] : dxh[t];
                const uint64_t db = (p == 0) ? dwl : dwh;
#pragma unroll
                for (int kb = 0; kb < kD / 16; kb++) {
                  // +32 bytes per 16-element K step inside the 128-byte swizzle row
                  mma_f16(dt, da + 2 * kb, db + 2 * kb, idesc_f16(kTileM, kGroupN - 32 * kb), (p | kb) != 0);
                }
              }
            }
            mma_commit(&S.acc_full[ab][t]);
          }
          if (!ok) break;
          mma_commit(&S.w_empty[ws]);
          wi++;
          ai++;
        }
        if (!ok) break;
        mma_commit(&S.x_empty);
        xi++;
      }
      // every MMA issued must complete before TMEM is released
      mma_commit(&S.mma_done);
      mbar_wait_drain(&S.mma_done, 0);
    }
  } else {
    // ------------------------------------------------ epilogue
    // 8 warps: warp w reads TMEM lanes 32 (w % 4) .. +31 of tile (w - 2) / 4
    const int quad = warp & 3;
    const int tile = (warp - 2) >> 2;
    const int row = quad * 32 + lane;
    const int prow = tile * kTileM + row;                 // point within the pair
    const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
    // l_ij scratch of this CTA: [pair parity][component][256 points of the pair]
    float *scr = lsc + (size_t)blockIdx.x * 2 * K * (2 * kTileM) + prow;
    double lsum = 0.0;
    bool ok = true;
    bool have_prev = false;
    int prev_par = 0;
    int64_t prev_i = -1;
    float prev_lse = 0.f;
    uint32_t ai = 0;
    int pc = 0;
    for (int64_t pr = blockIdx.x; pr < npairs && ok; pr += gridDim.x, pc++) {
      const int par = pc & 1;
      const bool live = tile < ((2 * pr + 1 < ntiles) ? 2 : 1);   // warp-uniform
      const int64_t pi = (live && (2 * pr + tile) * kTileM + row < n) ? (2 * pr + tile) * kTileM + row : -1;
      float mx = -INFINITY, se = 0.f, smax = 0.f;
      int jmax = 0;
      for (int g = 0; g < G; g++) {
        // posteriors of components 2g, 2g+1 of the previous pair: load early
        float lp[2] = {0.f, 0.f};
        if (have_prev && prev_i >= 0) {
#pragma unroll
          for (int q = 0; q < 2; q++) lp[q] = scr[(size_t)(prev_par * K + 2 * g + q) * (2 * kTileM)];
        }
        const int ab = ai & 1;
        if (!(ok = mbar_wait_warp(&S.acc_full[ab][tile], (ai >> 1) & 1, err))) break;
        tc_fence_after();
        float s[kCompPerGroup] = {0.f, 0.f};
        if (live) {
          const float *bg = S.bias + g * kGroupN;
          // 32-column block bp holds k-block (3 - bp) of both components:
          // column 32 bp + 16 q + t belongs to component q; two 64-column
          // loads per group, column pairs in packed FP32 arithmetic
          float2 s2[kCompPerGroup] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll 1
          for (int hp = 0; hp < kGroupN / 64; hp++) {
            uint32_t v[64];
            tmem_ld64(tbase + lane_addr + (2 * ab + tile) * kGroupN + hp * 64, v);
            tmem_wait_ld();
            const float4 *b4 = reinterpret_cast<const float4 *>(bg + hp * 64);
#pragma unroll
            for (int u = 0; u < 16; u++) {
              const float4 b = b4[u];
              const int q = (u >> 2) & 1;         // columns 4u .. 4u + 3
              const float2 y0 = __fadd2_rn(make_float2(__uint_as_float(v[4 * u]), __uint_as_float(v[4 * u + 1])),
                                           make_float2(-b.x, -b.y));
              const float2 y1 = __fadd2_rn(make_float2(__uint_as_float(v[4 * u + 2]), __uint_as_float(v[4 * u + 3])),
                                           make_float2(-b.z, -b.w));
              s2[q] = __ffma2_rn(y0, y0, s2[q]);
              s2[q] = __ffma2_rn(y1, y1, s2[q]);
            }
          }
          s[0] = s2[0].x + s2[0].y;
          s[1] = s2[1].x + s2[1].y;
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&S.acc_empty[ab][tile]);
        ai++;
        if (have_prev && prev_i >= 0) {
#pragma unroll
          for (int q = 0; q < 2; q++) store_post(Rh, Rl, (size_t)(2 * g + q) * np + prev_i, expf(lp[q] - prev_lse));
        }
        if (live) {
#pragma unroll
          for (int q = 0; q < kCompPerGroup; q++) {
            const int j = g * kCompPerGroup + q;
            // c_j carried as float hi + lo: its rounding would shift every
            // posterior of component j by the same factor
            const float l = (S.chi[j] - 0.5f * s[q]) + S.clo[j];
            scr[(size_t)(par * K + j) * (2 * kTileM)] = l;
            if (l > mx) {
              se = se * __expf(mx - l) + 1.f;
              mx = l;
              jmax = j;
              smax = s[q];
            } else if (l > -INFINITY) {
              se += __expf(l - mx);
            }
          }
        }
      }
      if (!ok) break;
      prev_i = pi;
      prev_lse = mx + __logf(se);
      if (pi >= 0) lsum += c64[jmax] - 0.5 * (double)smax + (double)__logf(se);
      prev_par = par;
      have_prev = true;
    }
    // posteriors of the last pair
    if (ok && have_prev && prev_i >= 0) {
      for (int j0 = 0; j0 < K; j0 += 8) {
        float l8[8];
#pragma unroll
        for (int u = 0; u < 8; u++)
          l8[u] = (j0 + u < K) ? scr[(size_t)(prev_par * K + j0 + u) * (2 * kTileM)] : 0.f;
#pragma unroll
        for (int u = 0; u < 8; u++)
          if (j0 + u < K) store_post(Rh, Rl, (size_t)(j0 + u) * np + prev_i, expf(l8[u] - prev_lse));
      }
    }
    // deterministic reduction over the 256 epilogue threads
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
    if (lane == 0) S.red[warp - 2] = lsum;
    asm volatile("bar.sync 1, 256;" ::: "memory");
    if (threadIdx.x == 64) {
      double t = 0.0;
      for (int w = 0; w < 8; w++) t += S.red[w];
      part[blockIdx.x] = t;
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tbase, 512);
}

// =============================================================== means
// Per 64-point block: D[128 comps x 80] += Rh Bh^T + Rh Bl^T + Rl Bh^T with
// B rows 0..63 = X^T (hi / lo) and row 64 of Bh = 1 (gives sum_i r_ij).
// Four epilogue warps flush the FP32 accumulator to FP64 partials every
// kFlushBlocks blocks (double-buffered TMEM, 2 x 128 columns).
__global__ void __launch_bounds__(192, 1)
k_means_tc(const __grid_constant__ CUtensorMap tm_rh, const __grid_constant__ CUtensorMap tm_rl,
           const __grid_constant__ CUtensorMap tm_xht, const __grid_constant__ CUtensorMap tm_xlt,
           int64_t n, double *__restrict__ part, int *err) {
  extern __shared__ uint8_t smem_raw[];
  MSmem &S = smem_aligned<MSmem>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nblocks = (n + kBlk - 1) / kBlk;
  // blocks of this CTA: b = blockIdx.x + t * gridDim.x, t < mine
  const int64_t mine = nblocks > blockIdx.x ? (nblocks - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int64_t nwin = (mine + kFlushBlocks - 1) / kFlushBlocks;

  // constant rows 64..79 of the B tiles (row 64 of Bh = ones; the rest zero);
  // rows of 128 bytes, 16-byte chunk c of row r stored at c ^ (r & 7)
  for (int e = threadIdx.x; e < kMStages * 16 * kBlk; e += blockDim.x) {
    const int s = e / (16 * kBlk), rem = e - s * 16 * kBlk;
    const int r = 64 + rem / kBlk, col = rem % kBlk;   // logical (row, point)
    const int phys = r * kBlk + (((col >> 3) ^ (r & 7)) << 3) + (col & 7);
    S.bh[s][phys] = __float2half(r == 64 ? 1.f : 0.f);
    S.bl[s][phys] = __float2half(0.f);
  }
  fence_proxy_async_smem();
  if (threadIdx.x == 0) {
    for (int s = 0; s < kMStages; s++) mbar_init(&S.in_full[s], 1), mbar_init(&S.in_empty[s], 1);
    for (int s = 0; s < 2; s++) mbar_init(&S.acc_full[s], 1), mbar_init(&S.acc_empty[s], 4);
    mbar_init(&S.mma_done, 1);
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&S.tmem_base, 256);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tmem_base;
  constexpr uint32_t kInBytes = 2 * kMaxK * kBlk * 2 + 2 * kD * kBlk * 2;

  if (warp == 0) {
    if (elect_one()) {
      bool ok = true;
      for (int64_t t = 0; t < mine && ok; t++) {
        const int s = (int)(t % kMStages);
        if (!(ok = mbar_wait_lazy(&S.in_empty[s], ((t / kMStages) & 1) ^ 1, err, 128))) break;
        const int p0 = (int)((blockIdx.x + t * gridDim.x) * kBlk);
        mbar_expect_tx(&S.in_full[s], kInBytes);
        tma_load_2d(S.rh[s], &tm_rh, &S.in_full[s], p0, 0);
        tma_load_2d(S.rl[s], &tm_rl, &S.in_full[s], p0, 0);
        tma_load_2d(S.bh[s], &tm_xht, &S.in_full[s], p0, 0);
        tma_load_2d(S.bl[s], &tm_xlt, &S.in_full[s], p0, 0);
      }
      for (int64_t u = mine - 1; u >= 0 && u >= mine - kMStages; u--)
        mbar_wait_drain(&S.in_full[u % kMStages], (u / kMStages) & 1);
    }
  } else if (warp == 1) {
    if (elect_one()) {
      bool ok = true;
      for (int64_t w = 0; w < nwin && ok; w++) {
        const int ab = w & 1;
        if (!(ok = mbar_wait(&S.acc_empty[ab], ((w >> 1) & 1) ^ 1, err))) break;
        const int64_t t1 = std::min<int64_t>(mine, (w + 1) * kFlushBlocks);
        for (int64_t t = w * kFlushBlocks; t < t1; t++) {
          const int s = (int)(t % kMStages);
          if (!(ok = mbar_wait(&S.in_full[s], (t / kMStages) & 1, err))) break;
          tc_fence_after();
          const uint64_t drh = sdesc_sw128(smem_u32(S.rh[s])), drl = sdesc_sw128(smem_u32(S.rl[s]));
          const uint64_t dbh = sdesc_sw128(smem_u32(S.bh[s])), dbl = sdesc_sw128(smem_u32(S.bl[s]));
#pragma unroll
          for (int p = 0; p < 3; p++) {
            const uint64_t da = (p == 2) ? drl : drh;
            const uint64_t db = (p == 1) ? dbl : dbh;
#pragma unroll
            for (int kb = 0; kb < kBlk / 16; kb++)
              mma_f16(tbase + ab * 128, da + 2 * kb, db + 2 * kb, idesc_f16(128, kMeanN),
                      (t != w * kFlushBlocks) || p || kb);
          }
          mma_commit(&S.in_empty[s]);
        }
        if (!ok) break;
        mma_commit(&S.acc_full[ab]);
      }
      mma_commit(&S.mma_done);
      mbar_wait_drain(&S.mma_done, 0);
    }
  } else {
    // flush: lane row = component; 80 columns -> this CTA's FP64 partial,
    // column-major (column c of component comp at o[c * kMaxK]) so a warp's
    // 32 components are 256 contiguous bytes
    const int quad = warp & 3;
    const int comp = quad * 32 + lane;
    double *o = part + (size_t)blockIdx.x * kMaxK * kMeanN + comp;
    for (int c = 0; c < kMeanN; c++) o[(size_t)c * kMaxK] = 0.0;
    bool ok = true;
    for (int64_t w = 0; w < nwin && ok; w++) {
      const int ab = w & 1;
      if (!(ok = mbar_wait_lazy_warp(&S.acc_full[ab], (w >> 1) & 1, err, 1000))) break;
      tc_fence_after();
      const uint32_t ta = tbase + ((uint32_t)(quad * 32) << 16) + ab * 128;
#pragma unroll 1
      for (int c0 = 0; c0 < 96; c0 += 32) {   // columns 80..95 are not used
        uint32_t v[32];
        tmem_ld32(ta + c0, v);
        tmem_wait_ld();
#pragma unroll
        for (int c = 0; c < 32; c++)
          if (c0 + c < kMeanN) o[(size_t)(c0 + c) * kMaxK] += (double)__uint_as_float(v[c]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.acc_empty[ab]);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tbase, 256);
}

// S1 = sum r, mu = S2 / S1, pi = S1 / N (FP64, blocks summed in order)
__global__ void k_final_means_tc(const double *__restrict__ part, int G, int K, int d, int64_t n,
                                 double *__restrict__ mu, double *__restrict__ pi,
                                 double *__restrict__ psum, float *__restrict__ muf) {
  const int j = blockIdx.x;
  __shared__ double s1;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int g = 0; g < G; g++) s += part[((size_t)g * kMeanN + kD) * kMaxK + j];
    s1 = s;
    psum[j] = s;
    pi[j] = s / (double)n;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < kD; q += blockDim.x) {
    double s = 0.0;
    for (int g = 0; g < G; g++) s += part[((size_t)g * kMeanN + q) * kMaxK + j];
    const double m = s / s1;
    if (q < d) mu[(size_t)j * d + q] = m;
    muf[(size_t)j * kD + q] = q < d ? (float)m : 0.f;
  }
}

// ========================================================= covariances
// CTA (blockIdx.x = group of 4 components, blockIdx.y = chunk of points).
// Producers (warps 2..17) form two groups of eight that take alternate
// blocks.  Warp c8 of a group owns the block's points 8 c8 .. 8 c8 + 7; lane a
// owns dimensions a and a + 32 (32 apart, so the eight rows a phase of a
// 16-byte store touches fall in eight different swizzle chunks).  For each of
// the 4 components q a thread writes z = sqrt(r) (x - mu) of its 8 points as
// one 16-byte store into rows (q % 2) * 64 + a (+ 32) of pair q / 2's operand
// tile and sums z^2 in FP32 / FP64 for the exact diagonal.
__global__ void __launch_bounds__(kCThreads, 1)
k_cov_tc(const __grid_constant__ CUtensorMap tm_x32, const __grid_constant__ CUtensorMap tm_rh4,
         const __grid_constant__ CUtensorMap tm_rl4, const float *__restrict__ muf, int64_t n,
         int64_t blocks_per_chunk, double *__restrict__ cpart, double *__restrict__ dpart, int *err) {
  extern __shared__ uint8_t smem_raw[];
  CSmem &S = smem_aligned<CSmem>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cg = blockIdx.x;                  // component group (4 components)
  const int64_t nblocks = (n + kBlk - 1) / kBlk;
  const int64_t b0 = (int64_t)blockIdx.y * blocks_per_chunk;
  const int64_t mine = std::max<int64_t>(0, std::min<int64_t>(nblocks, b0 + blocks_per_chunk) - b0);
  const int64_t nwin = (mine + kFlushBlocks - 1) / kFlushBlocks;
  const size_t cta = (size_t)blockIdx.y * gridDim.x + blockIdx.x;

  if (threadIdx.x == 0) {
    // each block is produced by one group of kCProd / 2 warps
    for (int s = 0; s < kCIn; s++) mbar_init(&S.in_full[s], 1), mbar_init(&S.in_empty[s], kCProd / 2);
    for (int s = 0; s < kZStages; s++) mbar_init(&S.z_full[s], kCProd / 2), mbar_init(&S.z_empty[s], 1);
    for (int s = 0; s < 2; s++) mbar_init(&S.acc_full[s], 1), mbar_init(&S.acc_empty[s], 4);
    mbar_init(&S.mma_done, 1);
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&S.tmem_base, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tmem_base;
  constexpr uint32_t kInBytes = kBlk * kD * 4 + 2 * 4 * kBlk * 2;

  if (warp == 0) {
    if (elect_one()) {
      bool ok = true;
      for (int64_t t = 0; t < mine && ok; t++) {
        const int s = (int)(t % kCIn);
        if (!(ok = mbar_wait_lazy(&S.in_empty[s], ((t / kCIn) & 1) ^ 1, err, 128))) break;
        const int p0 = (int)((b0 + t) * kBlk);
        mbar_expect_tx(&S.in_full[s], kInBytes);
        tma_load_2d(S.xs[s], &tm_x32, &S.in_full[s], 0, p0);
        tma_load_2d(S.rh[s], &tm_rh4, &S.in_full[s], p0, cg * 4);
        tma_load_2d(S.rl[s], &tm_rl4, &S.in_full[s], p0, cg * 4);
      }
      for (int64_t u = mine - 1; u >= 0 && u >= mine - kCIn; u--)
        mbar_wait_drain(&S.in_full[u % kCIn], (u / kCIn) & 1);
    }
  } else if (warp == 1) {
    if (elect_one()) {
      bool ok = true;
      constexpr uint32_t idesc = idesc_f16(128, 128);
      for (int64_t w = 0; w < nwin && ok; w++) {
        const int ab = w & 1;
        if (!(ok = mbar_wait(&S.acc_empty[ab], ((w >> 1) & 1) ^ 1, err))) break;
        const int64_t t1 = std::min<int64_t>(mine, (w + 1) * kFlushBlocks);
        for (int64_t t = w * kFlushBlocks; t < t1; t++) {
          const int s = (int)(t % kZStages);
          if (!(ok = mbar_wait(&S.z_full[s], (t / kZStages) & 1, err))) break;
          tc_fence_after();
#pragma unroll
          for (int pr = 0; pr < 2; pr++) {
            const uint64_t dz = sdesc_sw128(smem_u32(S.z[s][pr]));
#pragma unroll
            for (int kb = 0; kb < kBlk / 16; kb++)
              mma_f16(tbase + ab * 256 + pr * 128, dz + 2 * kb, dz + 2 * kb, idesc,
                      (t != w * kFlushBlocks) || kb);
          }
          mma_commit(&S.z_empty[s]);
        }
        if (!ok) break;
        mma_commit(&S.acc_full[ab]);
      }
      mma_commit(&S.mma_done);
      mbar_wait_drain(&S.mma_done, 0);
    }
  } else if (warp < 2 + kCProd) {
    // ------------------------------------------------ producers
    const int pw = warp - 2, grp = pw >> 3, c8 = pw & 7;
    const int a = lane;                          // dimensions a and a + 32
    float *srw = S.sr[pw];
    float2 nmu[4][2];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const float m = muf[(size_t)(cg * 4 + q) * kD + a + 32 * h];
        nmu[q][h] = make_float2(-m, -m);
      }
    double diag[4][2];
    float2 dwin[4][2];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int h = 0; h < 2; h++) diag[q][h] = 0.0, dwin[q][h] = make_float2(0.f, 0.f);
    bool ok = true;
    int li = 0;                                  // blocks this group has produced
    for (int64_t tb = grp; tb < mine && ok; tb += 2, li++) {
      const int si = (int)(tb % kCIn), sz = (int)(tb % kZStages);
      if (!(ok = mbar_wait_warp(&S.in_full[si], (tb / kCIn) & 1, err))) break;
      {
        // lane -> component lane / 8, point c8 * 8 + lane % 8; rows past N
        // read zero-filled r and x, and get s = 0 besides
        const int q = lane >> 3, p = c8 * 8 + (lane & 7);
        const float r = __half2float(S.rh[si][q * kBlk + p]) + __half2float(S.rl[si][q * kBlk + p]);
        const float sv = ((b0 + tb) * kBlk + p < n) ? sqrtf(r) : 0.f;
        __syncwarp();                           // the previous block's reads of the slot are done
        srw[lane] = sv;
        __syncwarp();
      }
      const float *xr = S.xs[si] + (c8 * 8) * kD + a;
      float2 xv[2][4];                           // [dimension a / a + 32][point pair]
#pragma unroll
      for (int h = 0; h < 2; h++)
#pragma unroll
        for (int u = 0; u < 4; u++) xv[h][u] = make_float2(xr[(2 * u) * kD + 32 * h], xr[(2 * u + 1) * kD + 32 * h]);
      if (!(ok = mbar_wait_warp(&S.z_empty[sz], ((tb / kZStages) & 1) ^ 1, err))) break;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const float4 s0 = *reinterpret_cast<const float4 *>(srw + q * 8);
        const float4 s1 = *reinterpret_cast<const float4 *>(srw + q * 8 + 4);
        const float2 s2[4] = {make_float2(s0.x, s0.y), make_float2(s0.z, s0.w), make_float2(s1.x, s1.y),
                              make_float2(s1.z, s1.w)};
#pragma unroll
        for (int h = 0; h < 2; h++) {
          uint32_t w4[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const float2 z = __fmul2_rn(__fadd2_rn(xv[h][u], nmu[q][h]), s2[u]);
            dwin[q][h] = __ffma2_rn(z, z, dwin[q][h]);
            const __half2 hz = __floats2half2_rn(z.x, z.y);
            w4[u] = *reinterpret_cast<const uint32_t *>(&hz);
          }
          const int row = ((q & 1) << 6) + a + 32 * h;
          uint8_t *zrow = reinterpret_cast<uint8_t *>(S.z[sz][q >> 1]) + row * 128;
          *reinterpret_cast<uint4 *>(zrow + ((c8 ^ (row & 7)) << 4)) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
        }
      }
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&S.z_full[sz]);
        mbar_arrive(&S.in_empty[si]);
      }
      if ((li + 1) % (kFlushBlocks / 2) == 0) {
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
          for (int h = 0; h < 2; h++)
            diag[q][h] += (double)dwin[q][h].x + (double)dwin[q][h].y, dwin[q][h] = make_float2(0.f, 0.f);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int h = 0; h < 2; h++) diag[q][h] += (double)dwin[q][h].x + (double)dwin[q][h].y;
    // exact diagonal: group 0, then group 1 added, then the 8 point chunks in order
    if (grp == 0)
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int h = 0; h < 2; h++) S.dred[c8][q][a + 32 * h] = diag[q][h];
    asm volatile("bar.sync 2, %0;" ::"n"(kCProd * 32) : "memory");
    if (grp == 1)
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int h = 0; h < 2; h++) S.dred[c8][q][a + 32 * h] += diag[q][h];
    asm volatile("bar.sync 2, %0;" ::"n"(kCProd * 32) : "memory");
    if (grp == 0 && c8 == 0)
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
          double v = S.dred[0][q][a + 32 * h];
          for (int c = 1; c < 8; c++) v += S.dred[c][q][a + 32 * h];
          dpart[(cta * 4 + q) * kD + a + 32 * h] = v;
        }
  } else {
    // ------------------------------------------------ flush warps 18..21
    const int quad = warp & 3;
    const int lrow = quad * 32 + lane;          // TMEM lane = row of the pair tile
    const int half = lrow >> 6;                 // 0: first component of the pair, 1: second
    // this CTA's FP64 partials, column-major per pair: column c of pair pr at
    // o[pr][c * 128] (row lrow), so a warp's 32 rows are 256 contiguous bytes
    double *o[2];
#pragma unroll
    for (int pr = 0; pr < 2; pr++) {
      o[pr] = cpart + (cta * 2 + pr) * (size_t)(kD * 128) + lrow;
      for (int c = 0; c < kD; c++) o[pr][(size_t)c * 128] = 0.0;
    }
    bool ok = true;
    for (int64_t w = 0; w < nwin && ok; w++) {
      const int ab = w & 1;
      if (!(ok = mbar_wait_lazy_warp(&S.acc_full[ab], (w >> 1) & 1, err, 1000))) break;
      tc_fence_after();
#pragma unroll
      for (int pr = 0; pr < 2; pr++) {
#pragma unroll 1
        for (int c0 = 0; c0 < kD; c0 += 32) {   // 32-column chunks
          uint32_t v[32];
          tmem_ld32(tbase + ((uint32_t)(quad * 32) << 16) + ab * 256 + pr * 128 + half * 64 + c0, v);
          tmem_wait_ld();
#pragma unroll
          for (int c = 0; c < 32; c++) o[pr][(size_t)(c0 + c) * 128] += (double)__uint_as_float(v[c]);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.acc_empty[ab]);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tbase, 512);
}

// Covs_j = sym(S3_j) / S1_j with the exact diagonal (FP64, chunks in order)
__global__ void k_final_cov_tc(const double *__restrict__ cpart, const double *__restrict__ dpart, int gx,
                               int gy, int d, const double *__restrict__ psum, double *__restrict__ sigma) {
  const int j = blockIdx.x, grp = j / 4, q = j % 4;
  const double inv = 1.0 / psum[j];
  double *Sg = sigma + (size_t)j * d * d;
  for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
    const int a = e / d, b = e - a * d;
    if (b < a) continue;
    double s = 0.0;
    if (a == b) {
      for (int c = 0; c < gy; c++) s += dpart[(((size_t)c * gx + grp) * 4 + q) * kD + a];
    } else {
      // partials of CTA (chunk c, group grp): pair q / 2, rows (q % 2) * 64 + row, column-major
      for (int c = 0; c < gy; c++) {
        const double *P = cpart + (((size_t)c * gx + grp) * 2 + (q >> 1)) * (kD * 128) + (q & 1) * 64;
        s += 0.5 * (P[(size_t)b * 128 + a] + P[(size_t)a * 128 + b]);
      }
    }
    s *= inv;
    Sg[a * d + b] = s;
    Sg[b * d + a] = s;
  }
}

// ====================================================== covariances (z x^T)
// Sigma_j N_j = sum_i r_ij (x_i - mu_j)(x_i - mu_j)^T  (ComputeWeightedTempDataset
// + BlockCovariances, EM2/MatrixEM.cpp:53-67,90-99), around the NEW means, as
//   sum_i z_i x_i^T - (sum_i z_i) mu_j^T,   z_i = r_ij (x_i - mu_j),
// with x = xh + xl (the FP16 split of X) on the B side, shared by every
// component: the per-component operand z is formed once per (point,
// component) by CUDA cores and written straight into tensor memory as the A
// operand of an M = 128 (two components x 64 dimensions) MMA; B = [Xh^T; 1]
// (N = 80, the ones row gives sum z in column 64) and Xl^T (N = 64) come from
// global memory by TMA.  Every output element of an MMA is wanted (no
// cross-component blocks), and the subtraction of (sum z) mu^T uses the sums
// of the ROUNDED z, so FP16 rounding of z enters only as sum delta_i (x_i -
// mu)^T: unbiased, centred, no diagonal correction needed.
//
// CTA (blockIdx.x = group of 4 components = 2 pairs, blockIdx.y = chunk of
// 64-point blocks).  Warp 0: TMA; warp 1: MMA; warps 2..2+4 kZSets-1:
// producers in groups of 4 (group = (warp - 2) / 4; kZSplit groups share a
// block, each forming its own K steps, and the kZSets / kZSplit teams take
// alternate blocks, so a block's operand is ready after a fraction of one
// warp's work); a warp writes the TMEM lanes 32 (warp % 4) .. +31: dimension
// 32 (warp & 1) + lane of the component in slot (warp & 3) / 2 of both pairs.
// The last 4 warps flush the FP32 accumulators to FP64 partials every
// kFlushBlocks blocks (double buffered in TMEM).
__global__ void __launch_bounds__(kZThreads, 1)
k_cov_zx(const __grid_constant__ CUtensorMap tm_xht, const __grid_constant__ CUtensorMap tm_xlt,
         const __grid_constant__ CUtensorMap tm_rh4, const float *__restrict__ muf, int64_t n,
         int64_t blocks_per_chunk, double *__restrict__ cpart, int *err) {
  extern __shared__ uint8_t smem_raw[];
  ZSmem &S = smem_aligned<ZSmem>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cg = blockIdx.x;
  const int64_t nblocks = (n + kBlk - 1) / kBlk;
  const int64_t b0 = (int64_t)blockIdx.y * blocks_per_chunk;
  const int64_t mine = std::max<int64_t>(0, std::min<int64_t>(nblocks, b0 + blocks_per_chunk) - b0);
  const int64_t nwin = (mine + kFlushBlocks - 1) / kFlushBlocks;
  const size_t cta = (size_t)blockIdx.y * gridDim.x + blockIdx.x;

  // constant rows 64..79 of the Bh stages (row 64 ones, the rest zero);
  // 16-byte chunk c of row r stored at c ^ (r & 7)
  for (int e = threadIdx.x; e < kZIn * 16 * kBlk; e += blockDim.x) {
    const int st = e / (16 * kBlk), rem = e - st * 16 * kBlk;
    const int r = 64 + rem / kBlk, col = rem % kBlk;
    S.bh[st][r * kBlk + (((col >> 3) ^ (r & 7)) << 3) + (col & 7)] = __float2half(r == 64 ? 1.f : 0.f);
  }
  fence_proxy_async_smem();
  if (threadIdx.x == 0) {
    // a block is read by the MMA and by the kZSplit * 4 producer warps that form its operand
    for (int st = 0; st < kZIn; st++) mbar_init(&S.in_full[st], 1), mbar_init(&S.in_empty[st], 4 * kZSplit + 1);
    for (int st = 0; st < kZA; st++) mbar_init(&S.a_full[st], 4 * kZSplit), mbar_init(&S.a_empty[st], 1);
    for (int b = 0; b < 2; b++) mbar_init(&S.acc_full[b], 1), mbar_init(&S.acc_empty[b], 4);
    mbar_init(&S.mma_done, 1);
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&S.tmem_base, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tmem_base;
  constexpr uint32_t kInBytes = 2 * kD * kBlk * 2 + 4 * kBlk * 2;

  if (warp == 0) {
    // ------------------------------------------------ TMA
    if (elect_one()) {
      bool ok = true;
      for (int64_t t = 0; t < mine && ok; t++) {
        const int st = (int)(t % kZIn);
        if (!(ok = mbar_wait_lazy(&S.in_empty[st], ((t / kZIn) & 1) ^ 1, err, 128))) break;
        // CTAs of the same point chunk (one per component group) start kZStagger
        // blocks apart, so they do not all request the same tile at once
        const int64_t tb = (t + (int64_t)cg * kZStagger) % mine;
        const int p0 = (int)((b0 + tb) * kBlk);
        mbar_expect_tx(&S.in_full[st], kInBytes);
        tma_load_2d(S.bh[st], &tm_xht, &S.in_full[st], p0, 0);
        tma_load_2d(S.bl[st], &tm_xlt, &S.in_full[st], p0, 0);
        tma_load_2d(S.rh[st], &tm_rh4, &S.in_full[st], p0, cg * 4);
      }
      for (int64_t u = mine - 1; u >= 0 && u >= mine - kZIn; u--)
        mbar_wait_drain(&S.in_full[u % kZIn], (u / kZIn) & 1);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA
    if (elect_one()) {
      bool ok = true;
      constexpr uint32_t idh = idesc_f16(128, kZN), idl = idesc_f16(128, kD);
      for (int64_t w = 0; w < nwin && ok; w++) {
        const int ab = w & 1;
        if (!(ok = mbar_wait(&S.acc_empty[ab], ((w >> 1) & 1) ^ 1, err))) break;
        const int64_t t1 = std::min<int64_t>(mine, (w + 1) * kFlushBlocks);
        for (int64_t t = w * kFlushBlocks; t < t1 && ok; t++) {
          const int st = (int)(t % kZIn), sa = (int)(t % kZA);
          if (!(ok = mbar_wait(&S.in_full[st], (t / kZIn) & 1, err))) break;
          if (!(ok = mbar_wait(&S.a_full[sa], (t / kZA) & 1, err))) break;
          tc_fence_after();
          const uint64_t dbh = sdesc_sw128(smem_u32(S.bh[st])), dbl = sdesc_sw128(smem_u32(S.bl[st]));
#pragma unroll
          for (int kb = 0; kb < kBlk / 16; kb++) {
#pragma unroll
            for (int pr = 0; pr < 2; pr++) {
              const uint32_t dt = tbase + ab * 2 * kZDCol + pr * kZDCol;
              const uint32_t at = tbase + kZACol + sa * kZAStage + pr * (kBlk / 2) + kb * 8;
              // +32 bytes per 16-point K step inside the 128-byte swizzle row
              mma_f16_ta(dt, at, dbh + 2 * kb, idh, (t != w * kFlushBlocks) || kb);
              mma_f16_ta(dt, at, dbl + 2 * kb, idl, 1);
            }
          }
          mma_commit(&S.a_empty[sa]);
          mma_commit(&S.in_empty[st]);
        }
        if (!ok) break;
        mma_commit(&S.acc_full[ab]);
      }
      mma_commit(&S.mma_done);
      mbar_wait_drain(&S.mma_done, 0);
    }
  } else if (warp < 2 + 4 * kZSets) {
    // ------------------------------------------------ producers
    const int pw = warp - 2, grp = pw >> 2, quad = warp & 3;
    const int team = grp / kZSplit, part = grp % kZSplit;   // team: blocks; part: K steps within a block
    constexpr int kTeams = kZSets / kZSplit, kSteps = kBlk / 16 / kZSplit;
    const int slot = quad >> 1;                  // component slot within each pair
    const int a = 32 * (quad & 1) + lane;        // dimension = TMEM lane within the slot
    const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
    float mu[2];
#pragma unroll
    for (int pr = 0; pr < 2; pr++) mu[pr] = muf[(size_t)(cg * 4 + 2 * pr + slot) * kD + a];
    bool ok = true;
    for (int64_t t = team; t < mine && ok; t += kTeams) {
      const int st = (int)(t % kZIn), sa = (int)(t % kZA);
      if (!(ok = mbar_wait_warp(&S.in_full[st], (t / kZIn) & 1, err))) break;
      if (!(ok = mbar_wait_warp(&S.a_empty[sa], ((t / kZA) & 1) ^ 1, err))) break;
      tc_fence_after();
      const uint8_t *rowh = reinterpret_cast<const uint8_t *>(S.bh[st]) + a * 128;
      const uint8_t *rowl = reinterpret_cast<const uint8_t *>(S.bl[st]) + a * 128;
#pragma unroll 1
      for (int kb = part * kSteps; kb < (part + 1) * kSteps; kb++) {
        // x = xh + xl (exact in FP32) of the 16 points of this K step, dimension a
        float2 x[8];
#pragma unroll
        for (int hc = 0; hc < 2; hc++) {
          const int c = 2 * kb + hc, pc = (c ^ (a & 7)) << 4;
          const uint4 vh = *reinterpret_cast<const uint4 *>(rowh + pc);
          const uint4 vl = *reinterpret_cast<const uint4 *>(rowl + pc);
          const uint32_t wh[4] = {vh.x, vh.y, vh.z, vh.w}, wl[4] = {vl.x, vl.y, vl.z, vl.w};
#pragma unroll
          for (int q = 0; q < 4; q++)
            x[4 * hc + q] = __fadd2_rn(__half22float2(*reinterpret_cast<const __half2 *>(&wh[q])),
                                       __half22float2(*reinterpret_cast<const __half2 *>(&wl[q])));
        }
#pragma unroll
        for (int pr = 0; pr < 2; pr++) {
          // z = fp16(x - mu) * r_hi, two points per half2 (the posteriors' hi
          // part: an 11-bit weight, its rounding as random as z's own)
          const uint4 *r4 = reinterpret_cast<const uint4 *>(S.rh[st] + (2 * pr + slot) * kBlk + 16 * kb);
          const uint4 ra = r4[0], rb = r4[1];
          const uint32_t rw[8] = {ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z, rb.w};
          const float2 nm = make_float2(-mu[pr], -mu[pr]);
          uint32_t packed[8];
#pragma unroll
          for (int q = 0; q < 8; q++) {
            const float2 dz = __fadd2_rn(x[q], nm);
            const __half2 z = __hmul2(__floats2half2_rn(dz.x, dz.y), *reinterpret_cast<const __half2 *>(&rw[q]));
            packed[q] = *reinterpret_cast<const uint32_t *>(&z);
          }
          tmem_st8(tbase + lane_addr + kZACol + sa * kZAStage + pr * (kBlk / 2) + kb * 8, packed);
        }
      }
      tmem_wait_st();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&S.a_full[sa]);
        mbar_arrive(&S.in_empty[st]);
      }
    }
  } else {
    // ------------------------------------------------ flush warps
    const int quad = warp & 3;
    const int lrow = quad * 32 + lane;          // TMEM lane = row of the pair tile
    // this CTA's FP64 partials, column-major per pair: column c of pair pr
    // at o[pr][c * 128] (row lrow), so a warp's 32 rows are 256 contiguous bytes
    double *o[2];
#pragma unroll
    for (int pr = 0; pr < 2; pr++) {
      o[pr] = cpart + (cta * 2 + pr) * (size_t)(kZCols * 128) + lrow;
      for (int c = 0; c < kZCols; c++) o[pr][(size_t)c * 128] = 0.0;
    }
    bool ok = true;
    for (int64_t w = 0; w < nwin && ok; w++) {
      const int ab = w & 1;
      if (!(ok = mbar_wait_lazy_warp(&S.acc_full[ab], (w >> 1) & 1, err, 1000))) break;
      tc_fence_after();
#pragma unroll
      for (int pr = 0; pr < 2; pr++) {
        const uint32_t ta = tbase + ((uint32_t)(quad * 32) << 16) + ab * 2 * kZDCol + pr * kZDCol;
#pragma unroll 1
        for (int c0 = 0; c0 < kD; c0 += 16) {   // 16-column loads (the pair pitch is 80 columns)
          uint32_t v[16];
          tmem_ld16(ta + c0, v);
          tmem_wait_ld();
#pragma unroll
          for (int c = 0; c < 16; c++) o[pr][(size_t)(c0 + c) * 128] += (double)__uint_as_float(v[c]);
        }
        uint32_t v16[16];
        tmem_ld16(ta + kD, v16);
        tmem_wait_ld();
        o[pr][(size_t)kD * 128] += (double)__uint_as_float(v16[0]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.acc_empty[ab]);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tbase, 512);
}

// Sigma_j = sym(sum z x^T - (sum z) muf^T) / N_j - (mu - muf)(mu - muf)^T:
// the scatter around the FP32 means the producers used, moved to the FP64
// means; chunks summed in order (FP64)
__global__ void k_final_cov_zx(const double *__restrict__ cpart, int gx, int gy, int d,
                               const double *__restrict__ psum, const double *__restrict__ mu,
                               const float *__restrict__ muf, double *__restrict__ sigma) {
  const int j = blockIdx.x, grp = j / 4, c = j % 4, pr = c >> 1, slot = c & 1;
  __shared__ double sz[kD];                    // sum z of component j, per dimension
  __shared__ double dm[kD];                    // mu - muf
  for (int a = threadIdx.x; a < kD; a += blockDim.x) {
    double v = 0.0;
    for (int ch = 0; ch < gy; ch++)
      v += cpart[(((size_t)ch * gx + grp) * 2 + pr) * (kZCols * 128) + (size_t)kD * 128 + slot * 64 + a];
    sz[a] = v;
    dm[a] = a < d ? mu[(size_t)j * d + a] - (double)muf[(size_t)j * kD + a] : 0.0;
  }
  __syncthreads();
  const double inv = 1.0 / psum[j];
  double *Sg = sigma + (size_t)j * d * d;
  for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
    const int a = e / d, b = e - a * d;
    if (b < a) continue;
    double sab = 0.0, sba = 0.0;
    for (int ch = 0; ch < gy; ch++) {
      const double *P = cpart + (((size_t)ch * gx + grp) * 2 + pr) * (kZCols * 128) + slot * 64;
      sab += P[(size_t)b * 128 + a];
      sba += P[(size_t)a * 128 + b];
    }
    const double ca = sab - sz[a] * (double)muf[(size_t)j * kD + b];
    const double cb = sba - sz[b] * (double)muf[(size_t)j * kD + a];
    const double v = 0.5 * (ca + cb) * inv - dm[a] * dm[b];
    Sg[a * d + b] = v;
    Sg[b * d + a] = v;
  }
}

// ================================================= bounded-wait expiry
// The exit path every warp-specialised kernel here relies on, run on purpose:
// one CTA with the roles of those kernels, whose producer never delivers.
// Warp 1 allocates all 512 TMEM columns (as the E-step and covariance kernels
// do) and waits for a barrier nothing arrives on, with `budget` cycles: the
// wait runs out, sets the status word and returns false; its drain wait
// (which ignores the status word, as the drains before TMEM release do) runs
// out too.  Warps 2 and 3 wait, off the critical path, for a barrier warp 1
// would have completed; they leave because the status word is set, not by
// their own (long) budget.  Every warp then reaches the final barrier and
// warp 1 releases TMEM.  roles[0..3] record which waits gave up.
__global__ void __launch_bounds__(128, 1) k_wait_expiry(long long budget, int *err, int *roles) {
  __shared__ uint64_t full, done;
  __shared__ uint32_t tslot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    mbar_init(&full, 1);
    mbar_init(&done, 1);
    fence_mbar_init();
  }
  if (warp == 1) tmem_alloc(&tslot, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    if (mbar_wait_warp(&full, 0, err, budget)) {
      if (lane == 0) mbar_arrive(&done);
    } else if (lane == 0) {
      roles[0] = 1;
    }
    if (lane == 0 && !mbar_wait_drain(&full, 0, budget)) roles[1] = 1;
  } else if (warp >= 2) {
    if (!mbar_wait_lazy_warp(&done, 0, err, 200) && lane == 0) roles[warp] = 1;
  }
  // warp 0, the producer, delivers nothing
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tslot, 512);
}

// ================================================ operand preparation
// W = L^-1 (FP64) -> FP16 hi/lo in the permuted row order; b = L^-1 mu;
// row of (component j, output k) = group j/2, k-block position 3 - k/16,
// component j%2, k%16
__device__ __forceinline__ int w_row(int j, int k) {
  return (j / kCompPerGroup) * kGroupN + (kD / 16 - 1 - k / 16) * (16 * kCompPerGroup) +
         (j % kCompPerGroup) * 16 + (k & 15);
}

// Dimensions d..63 of a component with d < 64 get zero rows and columns
// (x and mu are zero there, so y = 0), components K..Kp-1 (padding to a
// multiple of 4) get W = 0 and a log coefficient of -inf (posterior 0).
__global__ void k_prep_w(const double *__restrict__ linv, const double *__restrict__ mu, int K, int d,
                         __half *__restrict__ Wh, __half *__restrict__ Wl, float *__restrict__ bias,
                         const double *__restrict__ logc, float *__restrict__ chi, float *__restrict__ clo) {
  const int j = blockIdx.x;
  const bool live = j < K;
  if (threadIdx.x == 0) {
    chi[j] = live ? (float)logc[j] : -INFINITY;
    clo[j] = live ? (float)(logc[j] - (double)(float)logc[j]) : 0.f;
  }
  for (int e = threadIdx.x; e < kD * kD; e += blockDim.x) {
    const int k = e / kD, m = e - k * kD;
    const int row = w_row(j, k);
    const double w = (live && k < d && m < d) ? linv[((size_t)j * d + k) * d + m] : 0.0;
    const __half h = __double2half(w);
    Wh[(size_t)row * kD + m] = h;
    Wl[(size_t)row * kD + m] = __double2half(w - (double)__half2float(h));
  }
  for (int k = threadIdx.x; k < kD; k += blockDim.x) {
    double b = 0.0;
    if (live && k < d)
      for (int m = 0; m <= k; m++) b += linv[((size_t)j * d + k) * d + m] * mu[(size_t)j * d + m];
    bias[w_row(j, k)] = (float)b;
  }
}

// x -> xh = fp16(x), xl = fp16(x - xh), row-major and transposed (d x np)
// (rows of d < 64 values are zero-padded to 64; X64 receives the padded FP32
// rows when it is not null)
__global__ void k_split_x(const float *__restrict__ X, int64_t n, int d, __half *__restrict__ Xh,
                          __half *__restrict__ Xl, __half *__restrict__ XhT, __half *__restrict__ XlT,
                          int64_t np, float *__restrict__ X64, float *__restrict__ amax) {
  __shared__ __half th[kD][65], tl[kD][65];
  float m = 0.f;
  const int64_t nt = (n + 63) / 64;
  for (int64_t tile = blockIdx.x; tile < nt; tile += gridDim.x) {
    const int64_t r0 = tile * 64;
    for (int e = threadIdx.x; e < 64 * kD; e += blockDim.x) {
      const int r = e / kD, c = e - r * kD;
      if (r0 + r < n) {
        const float x = c < d ? X[(r0 + r) * d + c] : 0.f;
        if (X64) X64[(r0 + r) * kD + c] = x;
        const __half h = __float2half_rn(x);
        const __half l = __float2half_rn(x - __half2float(h));
        Xh[(r0 + r) * kD + c] = h;
        Xl[(r0 + r) * kD + c] = l;
        th[c][r] = h;
        tl[c][r] = l;
        m = fmaxf(m, fabsf(x));
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * kD; e += blockDim.x) {
      const int c = e / 64, r = e - c * 64;
      if (r0 + r < n) {
        XhT[(size_t)c * np + r0 + r] = th[c][r];
        XlT[(size_t)c * np + r0 + r] = tl[c][r];
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int *>(amax), __float_as_int(m));
}

__global__ void k_reduce_parts(const double *__restrict__ part, int np, DevStatus *st,
                               const int *__restrict__ err) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < np; b++) s += part[b];
    st->logl = s;
    if (*err) st->timeout = 1;
  }
}

__global__ void k_flag_timeout(DevStatus *st, const int *__restrict__ err) {
  if (threadIdx.x == 0 && *err) st->timeout = 1;
}

// posteriors (hi + lo) -> n x K double rows
__global__ void k_post_rows_tc(const __half *__restrict__ Rh, const __half *__restrict__ Rl, int64_t np,
                               int K, int64_t r0, int64_t rows, double *__restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * K) return;
  const int64_t i = e / K;
  const int j = (int)(e - i * K);
  const size_t o = (size_t)j * np + r0 + i;
  out[e] = (double)__half2float(Rh[o]) + (double)__half2float(Rl[o]);
}

__global__ void k_classes_tc(const __half *__restrict__ Rh, const __half *__restrict__ Rl, int64_t np,
                             int64_t n, int K, int32_t *__restrict__ cls) {
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
static size_t esmem_bytes() { return sizeof(ESmem) + 1024; }
static size_t msmem_bytes() { return sizeof(MSmem) + 1024; }
static size_t csmem_bytes() { return sizeof(CSmem) + 1024; }
static size_t zsmem_bytes() { return sizeof(ZSmem) + 1024; }

static int fp16_map(CUtensorMap *m, const void *base, uint64_t cols, uint64_t rows, uint64_t pitch_elems,
                    uint32_t box_cols, uint32_t box_rows, CUtensorMapSwizzle swz) {
  return encode_tmap_2d(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, base, cols, rows, box_cols, box_rows, swz,
                        pitch_elems * 2);
}

// the covariance kernel works on groups of 4 components
// d <= 64 (zero-padded to 64) and K <= 128 (padded to a multiple of 4)
bool em_tc_supported(int d, int k) {
  return (d >= 1 && d <= kD && k >= 1 && k <= kMaxK) || em_wide_supported(d, k);
}

// The tensor-core covariance rounds z to FP16 once; that error averages out
// over the points of a component (relative ~2^-12 / sqrt(N_j)).  With fewer
// than 16384 points per component on average it would not, so such fits take
// the FP32 CUDA-core covariance (its cost is small at that size).
bool em_tc_small_components(int64_t n, int k, int d) { return d <= kD && n < (int64_t)16384 * k; }

// covariance kernel selection while both forms are compared (FEM_COV_KERNEL=zz
// selects the z z^T form)
static bool cov_zx_enabled() {
  static const bool zx = [] {
    const char *v = getenv("FEM_COV_KERNEL");
    return !(v && v[0] == 'z' && v[1] == 'z');
  }();
  return zx;
}

int em_tc_create(fem_em *h) {
  if (h->d > kD) return em_wide_create(h);
  TcEmPlan *p = new TcEmPlan();
  h->tc = p;
  const int K = (h->k + 3) / 4 * 4;     // kernels see K padded to a multiple of 4
  const int64_t n = h->n;
  p->kp = K;
  p->d = h->d;
  p->np = (n + 63) / 64 * 64;
  const int sms = sm_count();
  FEM_TRY(dalloc(&h->Xhi, (size_t)n * kD));
  FEM_TRY(dalloc(&h->Xlo, (size_t)n * kD));
  FEM_TRY(dalloc(&p->XhT, (size_t)kD * p->np));
  FEM_TRY(dalloc(&p->XlT, (size_t)kD * p->np));
  FEM_TRY(dalloc(&p->Rh, (size_t)K * p->np));
  FEM_TRY(dalloc(&p->Rl, (size_t)K * p->np));
  FEM_TRY(dalloc(&p->Wh, (size_t)K * kD * kD));
  FEM_TRY(dalloc(&p->Wl, (size_t)K * kD * kD));
  FEM_TRY(dalloc(&p->bias, (size_t)K * kD));
  FEM_TRY(dalloc(&p->clo, K));
  FEM_TRY(dalloc(&p->muf, (size_t)K * kD));
  FEM_TRY(dalloc(&p->chi, K));
  FEM_CUDA(cudaMemset(p->muf, 0, (size_t)K * kD * sizeof(float)));
  if (h->d < kD) FEM_TRY(dalloc(&p->X64, (size_t)n * kD));
  FEM_TRY(dalloc(&p->err, 1));
  FEM_CUDA(cudaMemset(p->err, 0, sizeof(int)));
  FEM_TRY(dalloc(&p->amax, 1));
  FEM_TRY(dalloc(&p->roles, 4));
  const int64_t npairs = ((n + kTileM - 1) / kTileM + 1) / 2;
  p->egrid = (int)std::min<int64_t>(sms, npairs);
  FEM_TRY(dalloc(&p->epart, p->egrid));
  FEM_TRY(dalloc(&p->lsc, (size_t)p->egrid * 2 * K * 2 * kTileM));
  const int64_t nblocks = (n + kBlk - 1) / kBlk;
  p->mgrid = (int)std::min<int64_t>(sms, nblocks);
  FEM_TRY(dalloc(&p->mpart, (size_t)p->mgrid * kMaxK * kMeanN));
  p->cgx = K / 4;
  p->cgy = (int)std::max<int64_t>(1, std::min<int64_t>(nblocks, (4 * sms + p->cgx - 1) / p->cgx));
  FEM_TRY(dalloc(&p->cpart, (size_t)p->cgx * p->cgy * std::max(4 * kD * kD, 2 * kZCols * 128)));
  FEM_TRY(dalloc(&p->dpart, (size_t)p->cgx * p->cgy * 4 * kD));
  // E-step operands
  FEM_TRY(fp16_map(&p->tm_xh, h->Xhi, kD, n, kD, kD, kTileM, CU_TENSOR_MAP_SWIZZLE_128B));
  FEM_TRY(fp16_map(&p->tm_xl, h->Xlo, kD, n, kD, kD, kTileM, CU_TENSOR_MAP_SWIZZLE_128B));
  FEM_TRY(fp16_map(&p->tm_wh, p->Wh, kD, (uint64_t)K * kD, kD, kD, kGroupN, CU_TENSOR_MAP_SWIZZLE_128B));
  FEM_TRY(fp16_map(&p->tm_wl, p->Wl, kD, (uint64_t)K * kD, kD, kD, kGroupN, CU_TENSOR_MAP_SWIZZLE_128B));
  // means operands: rows of np-pitched component-major / transposed arrays
  FEM_TRY(encode_tmap_2d(&p->tm_rh, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->Rh, (uint64_t)n, (uint64_t)K, kBlk,
                         kMaxK, CU_TENSOR_MAP_SWIZZLE_128B, (uint64_t)p->np * 2));
  FEM_TRY(encode_tmap_2d(&p->tm_rl, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->Rl, (uint64_t)n, (uint64_t)K, kBlk,
                         kMaxK, CU_TENSOR_MAP_SWIZZLE_128B, (uint64_t)p->np * 2));
  FEM_TRY(encode_tmap_2d(&p->tm_xht, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->XhT, (uint64_t)n, kD, kBlk, kD,
                         CU_TENSOR_MAP_SWIZZLE_128B, (uint64_t)p->np * 2));
  FEM_TRY(encode_tmap_2d(&p->tm_xlt, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->XlT, (uint64_t)n, kD, kBlk, kD,
                         CU_TENSOR_MAP_SWIZZLE_128B, (uint64_t)p->np * 2));
  // covariance operands (no swizzle: read by CUDA cores)
  FEM_TRY(encode_tmap_2d(&p->tm_x32, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, p->X64 ? p->X64 : h->X, kD, (uint64_t)n, kD,
                         kBlk,
                         CU_TENSOR_MAP_SWIZZLE_NONE, 0));
  FEM_TRY(encode_tmap_2d(&p->tm_rh4, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->Rh, (uint64_t)n, (uint64_t)K, kBlk, 4,
                         CU_TENSOR_MAP_SWIZZLE_NONE, (uint64_t)p->np * 2));
  FEM_TRY(encode_tmap_2d(&p->tm_rl4, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->Rl, (uint64_t)n, (uint64_t)K, kBlk, 4,
                         CU_TENSOR_MAP_SWIZZLE_NONE, (uint64_t)p->np * 2));
  FEM_CUDA(cudaFuncSetAttribute(k_estep_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esmem_bytes()));
  FEM_CUDA(cudaFuncSetAttribute(k_means_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msmem_bytes()));
  FEM_CUDA(cudaFuncSetAttribute(k_cov_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem_bytes()));
  FEM_CUDA(cudaFuncSetAttribute(k_cov_zx, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zsmem_bytes()));
  return FEM_OK;
}

void em_tc_destroy(fem_em *h) {
  em_wide_destroy(h);
  TcEmPlan *p = h->tc;
  if (!p) return;
  dfree(p->Wh);
  dfree(p->Wl);
  dfree(p->bias);
  dfree(p->clo);
  dfree(p->Rh);
  dfree(p->Rl);
  dfree(p->XhT);
  dfree(p->XlT);
  dfree(p->lsc);
  dfree(p->epart);
  dfree(p->mpart);
  dfree(p->cpart);
  dfree(p->dpart);
  dfree(p->muf);
  dfree(p->chi);
  dfree(p->X64);
  dfree(p->err);
  dfree(p->amax);
  dfree(p->roles);
  delete p;
  h->tc = nullptr;
}

int em_tc_upload(fem_em *h) {
  if (h->wide) return em_wide_upload(h);
  TcEmPlan *p = h->tc;
  float *amax = p->amax;
  FEM_CUDA(cudaMemsetAsync(amax, 0, sizeof(float), h->stream));
  const int blocks = (int)std::min<int64_t>(4 * sm_count(), (h->n + 63) / 64);
  k_split_x<<<blocks, 256, 0, h->stream>>>(h->X, h->n, h->d, h->Xhi, h->Xlo, p->XhT, p->XlT, p->np, p->X64, amax);
  float m = 0.f;
  cudaMemcpyAsync(&m, amax, sizeof(float), cudaMemcpyDeviceToHost, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    set_error("dataset split failed: %s", cudaGetErrorString(e));
    return FEM_ERR_CUDA;
  }
  if (!(m < 32768.f)) {
    set_error("mixed precision needs |x| < 32768 (FP16 operands); max |x| = %g", m);
    return FEM_ERR_UNSUPPORTED;
  }
  return FEM_OK;
}

int em_tc_prepare(fem_em *h) {
  if (h->wide) return em_wide_prepare(h);
  TcEmPlan *p = h->tc;
  k_prep_w<<<p->kp, 256, 0, h->stream>>>(h->linv, h->mu, h->k, h->d, p->Wh, p->Wl, p->bias, h->logc, p->chi,
                                         p->clo);
  FEM_CUDA(cudaGetLastError());
  h->launches += 1;
  return FEM_OK;
}

int em_tc_estep(fem_em *h) {
  if (h->wide) return em_wide_estep(h);
  TcEmPlan *p = h->tc;
  k_estep_tc<<<p->egrid, kEThreads, esmem_bytes(), h->stream>>>(
      p->tm_xh, p->tm_xl, p->tm_wh, p->tm_wl, p->bias, p->chi, p->clo, h->logc, p->lsc, p->Rh, p->Rl, p->np,
      p->epart, h->n, p->kp, p->err);
  FEM_CUDA(cudaGetLastError());
  k_reduce_parts<<<1, 32, 0, h->stream>>>(p->epart, p->egrid, h->dstat, p->err);
  FEM_CUDA(cudaGetLastError());
  h->launches += 2;
  return FEM_OK;
}

int em_tc_mstep(fem_em *h) {
  if (h->wide) return em_wide_mstep(h);
  TcEmPlan *p = h->tc;
  const int K = h->k;
  k_means_tc<<<p->mgrid, 192, msmem_bytes(), h->stream>>>(p->tm_rh, p->tm_rl, p->tm_xht, p->tm_xlt, h->n,
                                                           p->mpart, p->err);
  FEM_CUDA(cudaGetLastError());
  k_final_means_tc<<<K, 64, 0, h->stream>>>(p->mpart, p->mgrid, K, h->d, h->n, h->mu, h->pi, h->psum, p->muf);
  FEM_CUDA(cudaGetLastError());
  if (em_tc_small_components(h->n, h->k, h->d)) {
    timing_begin(h, 8);
    FEM_TRY(em_cov_hilo(h, p->Rh, p->Rl, p->np, p->muf, kD));
    timing_begin(h, 9);
    k_flag_timeout<<<1, 32, 0, h->stream>>>(h->dstat, p->err);
    h->launches += 3;
    return FEM_OK;
  }
  const int64_t nblocks = (h->n + kBlk - 1) / kBlk;
  const int64_t bpc = (nblocks + p->cgy - 1) / p->cgy;
  timing_begin(h, 8);
  if (cov_zx_enabled()) {
    k_cov_zx<<<dim3(p->cgx, p->cgy), kZThreads, zsmem_bytes(), h->stream>>>(p->tm_xht, p->tm_xlt, p->tm_rh4, p->muf,
                                                                           h->n, bpc, p->cpart, p->err);
    FEM_CUDA(cudaGetLastError());
    timing_begin(h, 9);
    k_final_cov_zx<<<K, 256, 0, h->stream>>>(p->cpart, p->cgx, p->cgy, h->d, h->psum, h->mu, p->muf, h->sigma);
  } else {
    k_cov_tc<<<dim3(p->cgx, p->cgy), kCThreads, csmem_bytes(), h->stream>>>(p->tm_x32, p->tm_rh4, p->tm_rl4, p->muf,
                                                                           h->n, bpc, p->cpart, p->dpart, p->err);
    FEM_CUDA(cudaGetLastError());
    timing_begin(h, 9);
    k_final_cov_tc<<<K, 256, 0, h->stream>>>(p->cpart, p->dpart, p->cgx, p->cgy, h->d, h->psum, h->sigma);
  }
  FEM_CUDA(cudaGetLastError());
  k_flag_timeout<<<1, 32, 0, h->stream>>>(h->dstat, p->err);
  h->launches += 5;
  return FEM_OK;
}

// a wait that ran out in an earlier call leaves the status word set; each new
// call starts from zero (the context itself stays usable: nothing faulted)
int em_tc_reset_err(fem_em *h) {
  if (h->wide) return em_wide_reset_err(h);
  FEM_CUDA(cudaMemsetAsync(h->tc->err, 0, sizeof(int), h->stream));
  return FEM_OK;
}

int em_tc_wait_selftest(fem_em *h, long long budget, int *roles) {
  TcEmPlan *p = h->tc;
  FEM_CUDA(cudaMemsetAsync(p->roles, 0, 4 * sizeof(int), h->stream));
  k_wait_expiry<<<1, 128, 0, h->stream>>>(budget, p->err, p->roles);
  FEM_CUDA(cudaGetLastError());
  k_flag_timeout<<<1, 32, 0, h->stream>>>(h->dstat, p->err);
  FEM_CUDA(cudaGetLastError());
  int r[4] = {0, 0, 0, 0};
  FEM_CUDA(cudaMemcpyAsync(r, p->roles, sizeof r, cudaMemcpyDeviceToHost, h->stream));
  FEM_CUDA(cudaStreamSynchronize(h->stream));
  *roles = (r[0] ? 1 : 0) | (r[1] ? 2 : 0) | (r[2] ? 4 : 0) | (r[3] ? 8 : 0);
  h->launches += 2;
  return FEM_OK;
}

int em_tc_post_rows(fem_em *h, int64_t r0, int64_t rows, double *dout) {
  if (h->wide) return em_wide_post_rows(h, r0, rows, dout);
  TcEmPlan *p = h->tc;
  const int64_t tot = rows * h->k;
  k_post_rows_tc<<<(unsigned)((tot + 255) / 256), 256, 0, h->stream>>>(p->Rh, p->Rl, p->np, h->k, r0, rows, dout);
  FEM_CUDA(cudaGetLastError());
  return FEM_OK;
}

void em_tc_posteriors(fem_em *h, const __half **rh, const __half **rl, int64_t *pitch) {
  if (h->wide) return em_wide_posteriors(h, rh, rl, pitch);
  *rh = h->tc->Rh;
  *rl = h->tc->Rl;
  *pitch = h->tc->np;
}

int em_tc_classes(fem_em *h, int32_t *dcls) {
  if (h->wide) return em_wide_classes(h, dcls);
  TcEmPlan *p = h->tc;
  k_classes_tc<<<(unsigned)((h->n + 255) / 256), 256, 0, h->stream>>>(p->Rh, p->Rl, p->np, h->n, h->k, dcls);
  FEM_CUDA(cudaGetLastError());
  return FEM_OK;
}

}  // namespace fem
