// em_tc.cu -- tcgen05 mixed-precision EM sweep for sm_103a.
//
// E-step (MatrixEMBase::BlockDensities + PostProcessDensityMatrix,
// EM2/MatrixEM.cpp:39-51,69-81) as ONE tensor-core GEMM of each 128-point
// tile against the stacked inverse Cholesky factors of all components:
//   Y = X W^T,  W = [L_1^-1; ...; L_K^-1]  (K*d x d),  y_jk = (L_j^-1 x)_k
// in FP16 x 3 (x = xh + xl, W = Wh + Wl: Xh Wh^T + Xh Wl^T + Xl Wh^T) with
// FP32 accumulation in TMEM.  The epilogue subtracts b_j = L_j^-1 mu_j,
// squares and sums each component's d columns, adds the log coefficient,
// keeps an online log-sum-exp per point and writes l_ij, then the
// posteriors r_ij = exp(l_ij - LSE_i).  The per-point log-likelihood is
// accumulated in FP64 with the FP64 log coefficient of the winning
// component (a float coefficient would bias every point of a component by
// the same rounding error).
//
// Within a group of 4 components the 256 accumulator columns are ordered
// by 16-wide k-block, highest first, so K-step kb (m in [16kb, 16kb+16))
// only needs the first 256-64kb columns: the lower-triangular structure of
// L^-1 skips 37.5% of the MMA work.
//
// Warp roles (192 threads, one CTA per SM, persistent over tiles):
//   warp 0      TMA producer (X tile pair per tile, W group pair per group)
//   warp 1      TMEM owner + single-thread MMA issuer
//   warps 2..5  epilogue, one TMEM lane (= one point) per thread
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
constexpr int kTileM = 128;              // points per tile
constexpr int kGroupN = 256;             // accumulator columns per component group
constexpr int kCompPerGroup = kGroupN / kD;
constexpr int kXStages = 2, kWStages = 2;
constexpr uint32_t kXBytes = kTileM * kD * 2;    // one FP16 X tile (16 KB)
constexpr uint32_t kWBytes = kGroupN * kD * 2;   // one FP16 W group (32 KB)
constexpr int kEThreads = 192;

struct __align__(1024) ESmem {
  __half xh[kXStages][kTileM * kD];
  __half xl[kXStages][kTileM * kD];
  __half wh[kWStages][kGroupN * kD];
  __half wl[kWStages][kGroupN * kD];
  uint64_t x_full[kXStages], x_empty[kXStages];
  uint64_t w_full[kWStages], w_empty[kWStages];
  uint64_t acc_full[2], acc_empty[2];
  uint64_t mma_done;
  uint32_t tmem_base;
  double red[4];
};

struct TcEmPlan {
  CUtensorMap tm_xh, tm_xl, tm_wh, tm_wl;
  __half *Wh = nullptr, *Wl = nullptr;  // (K*d) x d, permuted rows
  float *bias = nullptr;                // K*d, permuted
  double *epart = nullptr;              // per-CTA log-likelihood
  int *err = nullptr;                   // device status of the bounded waits
  int egrid = 0;
};

// ============================================================== E-step
__global__ void __launch_bounds__(kEThreads, 1)
k_estep_tc(const __grid_constant__ CUtensorMap tm_xh, const __grid_constant__ CUtensorMap tm_xl,
           const __grid_constant__ CUtensorMap tm_wh, const __grid_constant__ CUtensorMap tm_wl,
           const float *__restrict__ bias, const float *__restrict__ c32,
           const double *__restrict__ c64, float *__restrict__ R, double *__restrict__ part,
           int64_t n, int K, int *err) {
  extern __shared__ uint8_t smem_raw[];
  ESmem &S = *reinterpret_cast<ESmem *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int G = K / kCompPerGroup;
  const int64_t ntiles = (n + kTileM - 1) / kTileM;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kXStages; s++) mbar_init(&S.x_full[s], 1), mbar_init(&S.x_empty[s], 1);
    for (int s = 0; s < kWStages; s++) mbar_init(&S.w_full[s], 1), mbar_init(&S.w_empty[s], 1);
    for (int s = 0; s < 2; s++) mbar_init(&S.acc_full[s], 1), mbar_init(&S.acc_empty[s], 4);
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
      for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int xs = xi % kXStages;
        if (!(ok = mbar_wait(&S.x_empty[xs], ((xi / kXStages) & 1) ^ 1, err))) break;
        mbar_expect_tx(&S.x_full[xs], 2 * kXBytes);
        tma_load_2d(S.xh[xs], &tm_xh, &S.x_full[xs], 0, (int)(tile * kTileM));
        tma_load_2d(S.xl[xs], &tm_xl, &S.x_full[xs], 0, (int)(tile * kTileM));
        xi++;
        for (int g = 0; g < G; g++) {
          const int ws = wi % kWStages;
          if (!(ok = mbar_wait(&S.w_empty[ws], ((wi / kWStages) & 1) ^ 1, err))) break;
          mbar_expect_tx(&S.w_full[ws], 2 * kWBytes);
          tma_load_2d(S.wh[ws], &tm_wh, &S.w_full[ws], 0, g * kGroupN);
          tma_load_2d(S.wl[ws], &tm_wl, &S.w_full[ws], 0, g * kGroupN);
          wi++;
        }
      }
      // drain: the last loads must land before the CTA may exit
      for (int s = 0; s < kXStages && xi > (uint32_t)s; s++) {
        const uint32_t u = xi - 1 - s;
        mbar_wait_drain(&S.x_full[u % kXStages], (u / kXStages) & 1);
      }
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
      for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int xs = xi % kXStages;
        if (!(ok = mbar_wait(&S.x_full[xs], (xi / kXStages) & 1, err))) break;
        tc_fence_after();
        const uint64_t dxh = sdesc_sw128(smem_u32(S.xh[xs]));
        const uint64_t dxl = sdesc_sw128(smem_u32(S.xl[xs]));
        for (int g = 0; g < G; g++) {
          const int ws = wi % kWStages, ab = ai & 1;
          if (!(ok = mbar_wait(&S.acc_empty[ab], ((ai >> 1) & 1) ^ 1, err))) break;
          if (!(ok = mbar_wait(&S.w_full[ws], (wi / kWStages) & 1, err))) break;
          tc_fence_after();
          const uint64_t dwh = sdesc_sw128(smem_u32(S.wh[ws]));
          const uint64_t dwl = sdesc_sw128(smem_u32(S.wl[ws]));
          const uint32_t dt = tbase + ab * kGroupN;
#pragma unroll
          for (int p = 0; p < 3; p++) {
            const uint64_t da = (p == 2) ? dxl : dxh;
            const uint64_t db = (p == 1) ? dwl : dwh;
#pragma unroll
            for (int kb = 0; kb < kD / 16; kb++) {
              // +32 bytes per 16-element K step inside the 128-byte swizzle row
              mma_f16(dt, da + 2 * kb, db + 2 * kb, idesc_f16(kTileM, kGroupN - 64 * kb),
                      (p | kb) != 0);
            }
          }
          mma_commit(&S.w_empty[ws]);
          mma_commit(&S.acc_full[ab]);
          wi++;
          ai++;
        }
        mma_commit(&S.x_empty[xs]);
        xi++;
      }
      // every MMA issued must complete before TMEM is released
      mma_commit(&S.mma_done);
      mbar_wait_drain(&S.mma_done, 0);
    }
  } else {
    // ------------------------------------------------ epilogue
    const int quad = warp & 3;
    const int row = quad * 32 + lane;
    const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
    uint32_t ai = 0;
    double lsum = 0.0;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
      const int64_t i = tile * kTileM + row;
      const bool valid = i < n;
      float mx = -INFINITY, se = 0.f, smax = 0.f;
      int jmax = 0;
      for (int g = 0; g < G; g++) {
        const int ab = ai & 1;
        // warp-uniform outcome: the TMEM loads below are .sync.aligned
        if (!(ok = __all_sync(0xffffffffu, mbar_wait(&S.acc_full[ab], (ai >> 1) & 1, err)))) break;
        tc_fence_after();
        float s[kCompPerGroup] = {0.f, 0.f, 0.f, 0.f};
        const float *bg = bias + (size_t)g * kGroupN;
        // 64-column block bp holds k-block (3 - bp) of all 4 components:
        // column 64 bp + 16 q + t belongs to component q
#pragma unroll 1
        for (int bp = 0; bp < kGroupN / 64; bp++) {
          uint32_t v[2][32];
          tmem_ld32(tbase + lane_addr + ab * kGroupN + bp * 64, v[0]);
          tmem_ld32(tbase + lane_addr + ab * kGroupN + bp * 64 + 32, v[1]);
          const float4 *b4 = reinterpret_cast<const float4 *>(bg + bp * 64);
          float4 b[16];
#pragma unroll
          for (int t = 0; t < 16; t++) b[t] = __ldg(b4 + t);
          tmem_wait_ld();
#pragma unroll
          for (int t = 0; t < 64; t++) {
            const float bb = (t & 3) == 0 ? b[t >> 2].x : (t & 3) == 1 ? b[t >> 2].y
                           : (t & 3) == 2 ? b[t >> 2].z : b[t >> 2].w;
            const float y = __uint_as_float(v[t >> 5][t & 31]) - bb;
            s[t >> 4] = fmaf(y, y, s[t >> 4]);
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&S.acc_empty[ab]);
        ai++;
#pragma unroll
        for (int q = 0; q < kCompPerGroup; q++) {
          const int j = g * kCompPerGroup + q;
          const float l = __ldg(c32 + j) - 0.5f * s[q];
          if (valid) R[(size_t)j * n + i] = l;
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
      if (!ok) break;
      if (valid) {
        const float lse = mx + __logf(se);
        lsum += __ldg(c64 + jmax) - 0.5 * (double)smax + (double)__logf(se);
        for (int j = 0; j < K; j++) {
          float *p = R + (size_t)j * n + i;
          *p = __expf(*p - lse);
        }
      }
    }
    // deterministic reduction over the 128 epilogue threads
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
    if (lane == 0) S.red[quad] = lsum;
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (threadIdx.x == 64) part[blockIdx.x] = S.red[0] + S.red[1] + S.red[2] + S.red[3];
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tbase, 512);
}

// ================================================ operand preparation
// W = L^-1 (FP64) -> FP16 hi/lo in the permuted row order; b = L^-1 mu
__global__ void k_prep_w(const double *__restrict__ linv, const double *__restrict__ mu, int K,
                         __half *__restrict__ Wh, __half *__restrict__ Wl, float *__restrict__ bias) {
  const int j = blockIdx.x;
  const int g = j / kCompPerGroup, q = j % kCompPerGroup;
  for (int e = threadIdx.x; e < kD * kD; e += blockDim.x) {
    const int k = e / kD, m = e - k * kD;
    const int row = g * kGroupN + (kD / 16 - 1 - k / 16) * 64 + q * 16 + (k & 15);
    const double w = linv[(size_t)j * kD * kD + e];
    const __half h = __double2half(w);
    Wh[(size_t)row * kD + m] = h;
    Wl[(size_t)row * kD + m] = __double2half(w - (double)__half2float(h));
  }
  for (int k = threadIdx.x; k < kD; k += blockDim.x) {
    double b = 0.0;
    for (int m = 0; m <= k; m++) b += linv[(size_t)j * kD * kD + k * kD + m] * mu[(size_t)j * kD + m];
    const int row = g * kGroupN + (kD / 16 - 1 - k / 16) * 64 + q * 16 + (k & 15);
    bias[row] = (float)b;
  }
}

// x -> xh = fp16(x), xl = fp16(x - xh)
__global__ void k_split_x(const float *__restrict__ X, int64_t count, __half *__restrict__ Xh,
                          __half *__restrict__ Xl, float *__restrict__ amax) {
  float m = 0.f;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const float x = X[e];
    const __half h = __float2half_rn(x);
    Xh[e] = h;
    Xl[e] = __float2half_rn(x - __half2float(h));
    m = fmaxf(m, fabsf(x));
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

// ==================================================== host: tensor maps
static int encode_2d(CUtensorMap *m, const void *base, uint64_t cols, uint64_t rows, uint32_t box_cols,
                     uint32_t box_rows) {
  return encode_tmap_2d(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, base, cols, rows, box_cols, box_rows,
                        CU_TENSOR_MAP_SWIZZLE_128B);
}

static size_t esmem_bytes() { return sizeof(ESmem) + 1024; }

bool em_tc_supported(int d, int k) { return d == kD && k % kCompPerGroup == 0 && k <= 1024; }

int em_tc_create(fem_em *h) {
  TcEmPlan *p = new TcEmPlan();
  h->tc = p;
  const int K = h->k;
  const int64_t n = h->n;
  FEM_TRY(dalloc(&h->Xhi, (size_t)n * kD));
  FEM_TRY(dalloc(&h->Xlo, (size_t)n * kD));
  FEM_TRY(dalloc(&p->Wh, (size_t)K * kD * kD));
  FEM_TRY(dalloc(&p->Wl, (size_t)K * kD * kD));
  FEM_TRY(dalloc(&p->bias, (size_t)K * kD));
  FEM_TRY(dalloc(&p->err, 1));
  FEM_CUDA(cudaMemset(p->err, 0, sizeof(int)));
  p->egrid = (int)std::min<int64_t>(sm_count(), (n + kTileM - 1) / kTileM);
  FEM_TRY(dalloc(&p->epart, p->egrid));
  FEM_TRY(encode_2d(&p->tm_xh, h->Xhi, kD, (uint64_t)n, kD, kTileM));
  FEM_TRY(encode_2d(&p->tm_xl, h->Xlo, kD, (uint64_t)n, kD, kTileM));
  FEM_TRY(encode_2d(&p->tm_wh, p->Wh, kD, (uint64_t)K * kD, kD, kGroupN));
  FEM_TRY(encode_2d(&p->tm_wl, p->Wl, kD, (uint64_t)K * kD, kD, kGroupN));
  FEM_CUDA(cudaFuncSetAttribute(k_estep_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esmem_bytes()));
  // the M-step runs on the FP32 CUDA-core kernels
  h->mgrid = (int)std::min<int64_t>((int64_t)4 * sm_count(), (n + 31) / 32);
  FEM_TRY(dalloc(&h->mpart, (size_t)h->mgrid * K * (kD + 1)));
  int TB, nb, nblk;
  cov_geometry(kD, &TB, &nb, &nblk);
  const int gx = (K * nblk + 255) / 256;
  h->cchunks = (int)std::max<int64_t>(1, std::min<int64_t>((3 * sm_count() + gx - 1) / gx, (n + 31) / 32));
  FEM_TRY(dalloc(&h->cpart, (size_t)h->cchunks * K * nblk * TB * TB));
  return FEM_OK;
}

void em_tc_destroy(fem_em *h) {
  TcEmPlan *p = h->tc;
  if (!p) return;
  dfree(p->Wh);
  dfree(p->Wl);
  dfree(p->bias);
  dfree(p->epart);
  dfree(p->err);
  delete p;
  h->tc = nullptr;
}

int em_tc_upload(fem_em *h) {
  float *amax = nullptr;
  FEM_TRY(dalloc(&amax, 1));
  FEM_CUDA(cudaMemsetAsync(amax, 0, sizeof(float), h->stream));
  const int64_t count = h->n * kD;
  const int blocks = (int)std::min<int64_t>(4096, (count + 255) / 256);
  k_split_x<<<blocks, 256, 0, h->stream>>>(h->X, count, h->Xhi, h->Xlo, amax);
  float m = 0.f;
  cudaMemcpyAsync(&m, amax, sizeof(float), cudaMemcpyDeviceToHost, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  dfree(amax);
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
  TcEmPlan *p = h->tc;
  k_prep_w<<<h->k, 256, 0, h->stream>>>(h->linv, h->mu, h->k, p->Wh, p->Wl, p->bias);
  FEM_CUDA(cudaGetLastError());
  h->launches += 1;
  return FEM_OK;
}

int em_tc_estep(fem_em *h) {
  TcEmPlan *p = h->tc;
  k_estep_tc<<<p->egrid, kEThreads, esmem_bytes(), h->stream>>>(
      p->tm_xh, p->tm_xl, p->tm_wh, p->tm_wl, p->bias, (const float *)h->logcT, h->logc, (float *)h->R,
      p->epart, h->n, h->k, p->err);
  FEM_CUDA(cudaGetLastError());
  k_reduce_parts<<<1, 32, 0, h->stream>>>(p->epart, p->egrid, h->dstat, p->err);
  FEM_CUDA(cudaGetLastError());
  h->launches += 2;
  return FEM_OK;
}

int em_tc_mstep(fem_em *h) { return em_plain_mstep(h); }

}  // namespace fem
