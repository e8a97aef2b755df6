// km_tc.cu -- Lloyd k-means assignment as a tcgen05 GEMM plus argmin
// (NaiveKMA::ComputeMSEAndCorrect, Clust/KMAlgorithm.cpp:205-255, for d = 32).
//
// Distances are translation invariant, so both sides are first centred on
// the data mean g (x' = x - g in FP32, c' = c - g in FP64): the error terms
// below scale with ||x'|| ||c'||, not with the distance from the origin.
// For a tile of 128 points the tensor cores form x'.c'_j for all K <= 256
// centroids in FP32 (TMEM), from FP16 hi/lo splits of x' and c':
//   A row  = [xh | xl]            (64 halves, one 128-byte swizzled row)
//   B1 row = [ch | ch], B2 row = [cl | 0]
//   A.B2 + A.B1 = xh.cl + (xh + xl).ch
// (issued small products first, xh.ch last).  The epilogue forms
// v_j = ||c'_j||^2 - 2 x'.c'_j, keeps the two smallest, and accepts the best
// when it is separated from the runner-up by a rigorous bound on the error of
// v (split residuals, tensor-core accumulation, FP32 rounding); otherwise the
// row is re-decided over all centroids in FP64 difference form, index order,
// strict < -- the reference's rule, bit for bit.  Rows are then added to
// exact 64-bit fixed-point centroid sums in shared memory (as km.cu does),
// so the update is order independent.
//
// Warp roles (448 threads): 0 TMA, 1 MMA (TMEM owner), 2..5 operand
// producers (FP32 row -> [xh | xl], ||x||), 6..13 epilogue in two groups of
// four, one group per TMEM accumulator buffer (alternate tiles).
#include <cfloat>
#include <cmath>

#include "km_kernels.cuh"
#include "tc_ptx.cuh"

namespace fem {

using namespace tc;

namespace {

constexpr int kKmD = 32;                 // dimension handled here
constexpr int kKmTile = 128;             // points per tile (MMA M)
constexpr int kKmMaxK = 256;             // centroids (MMA N)
constexpr int kKmXStages = 3;
constexpr int kKmAStages = 2;
constexpr int kKmAccPitch = kKmD + 1;    // padded rows of the fixed-point sums
constexpr int kKmThreads = 14 * 32;
constexpr uint32_t kKmXBytes = kKmTile * kKmD * 4;       // 16 KB FP32 tile
// bound constants (see k_km_tc_prep)
constexpr float kKmRel = 1.8310546875e-4f;                // 2^-13 + 2^-14
constexpr float kKmAbs = 3.814697265625e-6f;              // 2^-18
constexpr float kKmPad = 3.0e38f;                         // v of padding centroids

struct __align__(1024) KmSmem {
  __half b1[kKmMaxK * 64];                 // [ch | ch]  (SW128)
  __half b2[kKmMaxK * 64];                 // [cl | 0]   (SW128)
  __half a[kKmAStages][kKmTile * 64];      // [xh | xl]  (SW128)
  float x[kKmXStages][kKmTile * kKmD];     // FP32 rows  (SW128, TMA)
  long long acc[kKmMaxK * kKmAccPitch];    // fixed-point sums
  float cn2[kKmMaxK], bc[kKmMaxK], ac[kKmMaxK];
  float bcmax, acmax;
  float g[kKmD];                           // data mean (FP32)
  float xn[kKmXStages][kKmTile];           // ||x|| of the rows of each X stage
  int cnt[kKmMaxK];
  uint64_t b_full, x_full[kKmXStages], x_empty[kKmXStages], a_full[kKmAStages], a_empty[kKmAStages],
      acc_full[2], acc_empty[2], mma_done;
  uint32_t tmem_base;
};
static_assert(sizeof(KmSmem) + 1024 <= 232448, "k-means kernel shared memory");

struct KmTcPlanImpl {
  CUtensorMap tm_x, tm_b1, tm_b2;
  __half *b1 = nullptr, *b2 = nullptr;   // Kp x 64
  float *cconst = nullptr;               // 3 x Kp: ||c||^2, bound slope, bound offset
  int *err = nullptr;
  int kp = 0;
};

__device__ __forceinline__ void fence_proxy_async_smem_km() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// centroid operands and bound constants (FP64 centroids in)
__global__ void k_km_tc_prep(const double *__restrict__ cent, const double *__restrict__ g, int K, int Kp,
                             __half *__restrict__ b1, __half *__restrict__ b2, float *__restrict__ cconst) {
  const int j = blockIdx.x, t = threadIdx.x;   // 64 threads: t < 32 hi / lo of dim t, t >= 32 copy of hi
  const int q = t & (kKmD - 1);
  __shared__ double red[64];
  const double c = j < K ? cent[(size_t)j * kKmD + q] - g[q] : 0.0;
  const __half ch = __double2half(c);
  const __half cl = __double2half(c - (double)__half2float(ch));
  b1[(size_t)j * 64 + t] = ch;                        // [ch | ch]
  b2[(size_t)j * 64 + t] = t < kKmD ? cl : __float2half(0.f);
  red[t] = t < kKmD ? c * c : 0.0;
  red[q] = q < kKmD ? c * c : 0.0;
  __syncthreads();
  if (t == 0) {
    double s = 0.0;
    for (int t = 0; t < kKmD; t++) s += red[t];
    const float n2 = (float)s, nrm = (float)sqrt(s);
    // |v_j - (||c'||^2 - 2 x'.c')| <= ||x'|| bc_j + ac_j + ax(||x'||)  (v in FP32);
    // 2^-14 ||x'|| ||c'|| + 2^-15 ||c'||^2 of it cover the centroid index kept
    // in the low 8 bits of the scanned values (at most 2^-15 |v|)
    cconst[j] = j < K ? n2 : kKmPad;
    cconst[Kp + j] = j < K ? kKmRel * nrm : 0.f;
    const float a = j < K ? kKmAbs * nrm + 3.147125244140625e-5f * n2 + 1e-30f : 0.f;   // 2^-15 + 2^-20
    cconst[2 * Kp + j] = a;
    // maxima over the centroids (non-negative floats order like their bits)
    atomicMax(reinterpret_cast<int *>(cconst + 3 * Kp), __float_as_int(cconst[Kp + j]));
    atomicMax(reinterpret_cast<int *>(cconst + 3 * Kp + 1), __float_as_int(a));
  }
}

// FP64 difference form in column order without contraction (the reference's
// per-point squared distance)
__device__ __forceinline__ double km_dist64(const double *__restrict__ c, const float *x) {
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < kKmD; q++) {
    const double t = __dsub_rn(c[q], (double)x[q]);
    s = __dadd_rn(s, __dmul_rn(t, t));
  }
  return s;
}

// FP32 difference form (as the FP32 path computes it) and a bound on its
// distance from the exact value, for rows the tensor-core screen leaves open
__device__ __forceinline__ float km_dist32(const float *__restrict__ c, const float *x) {
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < kKmD; q++) {
    const float t = x[q] - c[q];
    s = fmaf(t, t, s);
  }
  return s;
}
__device__ __forceinline__ float km_bound32(float s, float cn) {
  const float u = 5.9604645e-8f;  // 2^-24
  return 2.f * ((float)(kKmD + 4) * u * s + 2.01f * u * sqrtf(fmaxf(s, 0.f)) * cn + u * u * cn * cn) + 1e-30f;
}

// refinement state: the FP32 candidates' smallest upper bound and the two
// smallest lower bounds (with the index of the smallest)
struct KmRefine {
  float U = INFINITY, l1 = INFINITY, l2 = INFINITY;
  int j1 = 0;
  __device__ __forceinline__ void add(int j, const float *__restrict__ centf, const float *__restrict__ cnorm,
                                      const float *x) {
    const float s32 = km_dist32(centf + (size_t)j * kKmD, x);
    const float e = km_bound32(s32, cnorm[j]);
    U = fminf(U, s32 + e);
    const float lb = s32 - e;
    if (lb < l1) {
      l2 = l1;
      l1 = lb;
      j1 = j;
    } else {
      l2 = fminf(l2, lb);
    }
  }
  __device__ __forceinline__ bool decided() const { return l2 > U; }
};

__global__ void __launch_bounds__(kKmThreads, 1)
k_km_assign_tc(const __grid_constant__ CUtensorMap tm_x, const __grid_constant__ CUtensorMap tm_b1,
               const __grid_constant__ CUtensorMap tm_b2, const float *__restrict__ cconst,
               const double *__restrict__ cent, const float *__restrict__ centf,
               const float *__restrict__ cnorm, const double *__restrict__ gmean, int64_t n, int K, int Kp,
               int32_t *__restrict__ labels,
               long long *__restrict__ accg, int *__restrict__ cntg, float scale, DevStatus *st,
               int *err) {
  extern __shared__ uint8_t smem_raw[];
  KmSmem &S = smem_aligned<KmSmem>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ntiles = (n + kKmTile - 1) / kKmTile;
  const int64_t mine = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

  for (int e = threadIdx.x; e < kKmMaxK * kKmAccPitch; e += blockDim.x) S.acc[e] = 0;
  for (int j = threadIdx.x; j < kKmMaxK; j += blockDim.x) {
    S.cnt[j] = 0;
    S.cn2[j] = j < Kp ? cconst[j] : kKmPad;
    S.bc[j] = j < Kp ? cconst[Kp + j] : 0.f;
    S.ac[j] = j < Kp ? cconst[2 * Kp + j] : 0.f;
  }
  if (threadIdx.x < kKmD) S.g[threadIdx.x] = (float)gmean[threadIdx.x];
  if (threadIdx.x == 0) {
    S.bcmax = cconst[3 * Kp];
    S.acmax = cconst[3 * Kp + 1];
    mbar_init(&S.b_full, 1);
    for (int s = 0; s < kKmXStages; s++) mbar_init(&S.x_full[s], 1), mbar_init(&S.x_empty[s], 4);
    for (int s = 0; s < kKmAStages; s++) mbar_init(&S.a_full[s], 4), mbar_init(&S.a_empty[s], 1);
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
    // ------------------------------------------------ TMA
    if (elect_one()) {
      tma_prefetch_desc(&tm_x);
      mbar_expect_tx(&S.b_full, 2u * Kp * 128u);
      tma_load_2d(S.b1, &tm_b1, &S.b_full, 0, 0);
      tma_load_2d(S.b2, &tm_b2, &S.b_full, 0, 0);
      bool ok = true;
      for (int64_t i = 0; i < mine && ok; i++) {
        const int s = (int)(i % kKmXStages);
        if (!(ok = mbar_wait_lazy(&S.x_empty[s], ((i / kKmXStages) & 1) ^ 1, err, 64))) break;
        mbar_expect_tx(&S.x_full[s], kKmXBytes);
        tma_load_2d(S.x[s], &tm_x, &S.x_full[s], 0, (int)((blockIdx.x + i * gridDim.x) * kKmTile));
      }
      mbar_wait_drain(&S.b_full, 0);
      for (int64_t u = mine - 1; u >= 0 && u >= mine - kKmXStages; u--)
        mbar_wait_drain(&S.x_full[u % kKmXStages], (u / kKmXStages) & 1);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (elect_one()) {
      bool ok = mbar_wait(&S.b_full, 0, err);
      tc_fence_after();
      const uint64_t db1 = sdesc_sw128(smem_u32(S.b1)), db2 = sdesc_sw128(smem_u32(S.b2));
      const uint32_t idesc = idesc_f16(kKmTile, Kp);
      for (int64_t i = 0; i < mine && ok; i++) {
        const int as = (int)(i % kKmAStages), ab = (int)(i & 1);
        if (!(ok = mbar_wait(&S.acc_empty[ab], ((i >> 1) & 1) ^ 1, err))) break;
        if (!(ok = mbar_wait(&S.a_full[as], (i / kKmAStages) & 1, err))) break;
        tc_fence_after();
        const uint64_t da = sdesc_sw128(smem_u32(S.a[as]));
        const uint32_t d = tbase + ab * kKmMaxK;
        // xh.cl (k-blocks 0, 1 of B2), xl.ch (k-blocks 2, 3 of B1), xh.ch (0, 1 of B1)
        mma_f16(d, da + 0, db2 + 0, idesc, 0);
        mma_f16(d, da + 2, db2 + 2, idesc, 1);
        mma_f16(d, da + 4, db1 + 4, idesc, 1);
        mma_f16(d, da + 6, db1 + 6, idesc, 1);
        mma_f16(d, da + 0, db1 + 0, idesc, 1);
        mma_f16(d, da + 2, db1 + 2, idesc, 1);
        mma_commit(&S.a_empty[as]);
        mma_commit(&S.acc_full[ab]);
      }
      mma_commit(&S.mma_done);
      mbar_wait_drain(&S.mma_done, 0);
    }
  } else if (warp < 6) {
    // ------------------------------------------------ producers: row r
    const int r = (warp - 2) * 32 + lane;
    bool ok = true;
    for (int64_t i = 0; i < mine && ok; i++) {
      const int s = (int)(i % kKmXStages), as = (int)(i % kKmAStages);
      if (!(ok = mbar_wait_warp(&S.x_full[s], (i / kKmXStages) & 1, err))) break;
      if (!(ok = mbar_wait_warp(&S.a_empty[as], ((i / kKmAStages) & 1) ^ 1, err))) break;
      const float4 *xr = reinterpret_cast<const float4 *>(S.x[s] + r * kKmD);
      uint4 *ar = reinterpret_cast<uint4 *>(S.a[as] + r * 64);
      float ss = 0.f;
#pragma unroll
      for (int c2 = 0; c2 < 4; c2++) {          // 8 floats -> one 16-byte chunk of xh and of xl
        const float4 u = xr[(2 * c2) ^ (r & 7)];
        const float4 w = xr[(2 * c2 + 1) ^ (r & 7)];
        const float v[8] = {u.x - S.g[8 * c2], u.y - S.g[8 * c2 + 1], u.z - S.g[8 * c2 + 2],
                            u.w - S.g[8 * c2 + 3], w.x - S.g[8 * c2 + 4], w.y - S.g[8 * c2 + 5],
                            w.z - S.g[8 * c2 + 6], w.w - S.g[8 * c2 + 7]};
        uint32_t hh[4], ll[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const __half2 h = __floats2half2_rn(v[2 * e], v[2 * e + 1]);
          const float2 hf = __half22float2(h);
          const __half2 l = __floats2half2_rn(v[2 * e] - hf.x, v[2 * e + 1] - hf.y);
          hh[e] = *reinterpret_cast<const uint32_t *>(&h);
          ll[e] = *reinterpret_cast<const uint32_t *>(&l);
          ss = fmaf(v[2 * e], v[2 * e], ss);
          ss = fmaf(v[2 * e + 1], v[2 * e + 1], ss);
        }
        ar[c2 ^ (r & 7)] = make_uint4(hh[0], hh[1], hh[2], hh[3]);
        ar[(4 + c2) ^ (r & 7)] = make_uint4(ll[0], ll[1], ll[2], ll[3]);
      }
      // ||x'|| rounded up a little so that the bound stays an upper bound
      S.xn[s][r] = sqrtf(ss) * 1.00001f;
      fence_proxy_async_smem_km();
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.a_full[as]);
    }
  } else {
    // ------------------------------------------------ epilogue: group g, TMEM lanes of warp % 4
    const int g = (warp - 6) >> 2, quad = warp & 3;
    const int r = quad * 32 + lane;
    const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
    int64_t rechecks = 0;
    bool ok = true;
    for (int64_t i = g; i < mine && ok; i += 2) {
      const int s = (int)(i % kKmXStages);
      if (!(ok = mbar_wait_warp(&S.acc_full[g], (i >> 1) & 1, err))) break;
      tc_fence_after();
      // the three smallest v; the centroid index rides in the low 8 bits of
      // each value (v changes by at most 2^-15 |v|, which the bound covers),
      // so the scan is a min/max network without index bookkeeping
      float m1 = kKmPad, m2 = kKmPad, m3 = kKmPad;
      auto scan = [&](float v, int j) {
        const float e = __int_as_float((__float_as_int(v) & ~0xFF) | j);
        const float hi = fmaxf(m1, e);
        m1 = fminf(m1, e);
        const float hi2 = fmaxf(m2, hi);
        m2 = fminf(m2, hi);
        m3 = fminf(m3, hi2);
      };
      int c0 = 0;
#pragma unroll 1
      for (; c0 + 32 <= Kp; c0 += 32) {
        uint32_t dv[32];
        tmem_ld32(tbase + lane_addr + g * kKmMaxK + c0, dv);
        tmem_wait_ld();
#pragma unroll
        for (int t = 0; t < 32; t++) scan(fmaf(-2.f, __uint_as_float(dv[t]), S.cn2[c0 + t]), c0 + t);
      }
      if (c0 < Kp) {                             // Kp is a multiple of 16
        uint32_t dv[16];
        tmem_ld16(tbase + lane_addr + g * kKmMaxK + c0, dv);
        tmem_wait_ld();
#pragma unroll
        for (int t = 0; t < 16; t++) scan(fmaf(-2.f, __uint_as_float(dv[t]), S.cn2[c0 + t]), c0 + t);
      }
      const int j1 = __float_as_int(m1) & 0xFF, j2 = __float_as_int(m2) & 0xFF;
      const float v1 = m1, v2 = m2, v3 = m3;
      const int64_t row = (blockIdx.x + i * gridDim.x) * kKmTile + r;
      const float *xs = S.x[s] + r * kKmD;
      const float xn = S.xn[s][r];
      // 2^-18 ||x'|| for split residuals, 2^-23 ||x'||^2 for the rounding of x - g
      const float ax = fmaf(1.1920928955078125e-7f * xn, xn, kKmAbs * xn);
      const float b1 = fmaf(xn, S.bc[j1], S.ac[j1]) + ax;
      const float bmax = fmaf(xn, S.bcmax, S.acmax) + ax;   // >= every centroid's bound
      // the winner's exact distance is at most u; a centroid j with
      // v_j - bound_j > u cannot be the reference's choice
      const float u = v1 + b1;
      // 0: j1 is separated, 1: the candidates are j1 and j2, 2: more than two
      const int mode = (row >= n || v2 - bmax > u) ? 0 : (v3 - bmax > u ? 1 : 2);
      int lab = j1;
      float x[kKmD];
      if (mode != 0) {
#pragma unroll
        for (int q = 0; q < kKmD; q++) x[q] = xs[(((q >> 2) ^ (r & 7)) << 2) + (q & 3)];
      }
      // mode 2: FP32 difference form over the tensor-core candidates; rows it
      // cannot separate either go to FP64 over the same candidates (pass 3)
      bool fp64 = false;
      if (__any_sync(0xffffffffu, mode == 2)) {
        KmRefine rf;
#pragma unroll 1
        for (int c0 = 0; c0 < Kp; c0 += 32) {
          uint32_t dv[32];
          tmem_ld32(tbase + lane_addr + g * kKmMaxK + c0, dv);
          tmem_wait_ld();
          if (mode == 2) {
#pragma unroll 1
            for (int t = 0; t < 32; t++) {
              const int j = c0 + t;
              const float v = fmaf(-2.f, __uint_as_float(dv[t]), S.cn2[j]);
              if (j < K && v - (fmaf(xn, S.bc[j], S.ac[j]) + ax) <= u) rf.add(j, centf, cnorm, x);
            }
          }
        }
        if (mode == 2) {
          lab = rf.j1;
          fp64 = !rf.decided();
        }
        if (__any_sync(0xffffffffu, fp64)) {
          // the reference's FP64 decision (index order, strict <) over the candidates
          double best = DBL_MAX;
#pragma unroll 1
          for (int c0 = 0; c0 < Kp; c0 += 32) {
            uint32_t dv[32];
            tmem_ld32(tbase + lane_addr + g * kKmMaxK + c0, dv);
            tmem_wait_ld();
            if (fp64) {
#pragma unroll 1
              for (int t = 0; t < 32; t++) {
                const int j = c0 + t;
                const float v = fmaf(-2.f, __uint_as_float(dv[t]), S.cn2[j]);
                if (j < K && v - (fmaf(xn, S.bc[j], S.ac[j]) + ax) <= u) {
                  const double d64 = km_dist64(cent + (size_t)j * kKmD, x);
                  if (d64 < best) {
                    best = d64;
                    lab = j;
                  }
                }
              }
            }
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.acc_empty[g]);

      if (row < n) {
        if (mode != 0) rechecks++;
        if (mode == 1) {
          // two candidates: FP32 difference form, then the reference's FP64
          // comparison if that cannot separate them (lower index on ties)
          const int ja = min(j1, j2), jb = max(j1, j2);
          KmRefine rf;
          rf.add(ja, centf, cnorm, x);
          rf.add(jb, centf, cnorm, x);
          if (rf.decided()) {
            lab = rf.j1;
          } else {
            const double da = km_dist64(cent + (size_t)ja * kKmD, x);
            const double db = km_dist64(cent + (size_t)jb * kKmD, x);
            lab = db < da ? jb : ja;
          }
        }
        if (st->track_changes && labels[row] != lab) st->changed = 1;
        labels[row] = lab;
        atomicAdd(&S.cnt[lab], 1);
      }
      // exact fixed-point sums, one row of the warp at a time: lane q adds
      // dimension q, so each 64-bit atomic instruction updates 32 consecutive
      // words of one centroid row (conflict-free) instead of 32 scattered rows
      {
        const int mylab = row < n ? lab : -1;
#pragma unroll 4
        for (int rr = 0; rr < 32; rr++) {
          const int l = __shfl_sync(0xffffffffu, mylab, rr);
          if (l >= 0) {
            const int rq = quad * 32 + rr;
            const float xv = S.x[s][rq * kKmD + ((((lane >> 2) ^ (rq & 7)) << 2) + (lane & 3))];
            atomicAdd(reinterpret_cast<unsigned long long *>(S.acc + l * kKmAccPitch + lane),
                      (unsigned long long)__float2ll_rn(xv * scale));
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.x_empty[s]);
    }
    if (rechecks) atomicAdd((unsigned long long *)&st->rechecked, (unsigned long long)rechecks);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tbase, 512);
  // per-CTA partials in the layout k_km_final reads: [cta][j][q], [cta][j]
  for (int e = threadIdx.x; e < K * kKmD; e += blockDim.x) {
    const int j = e / kKmD, q = e - j * kKmD;
    accg[(size_t)blockIdx.x * K * kKmD + e] = S.acc[j * kKmAccPitch + q];
  }
  for (int j = threadIdx.x; j < K; j += blockDim.x) cntg[(size_t)blockIdx.x * K + j] = S.cnt[j];
}

__global__ void k_km_tc_flag(DevStatus *st, const int *__restrict__ err) {
  if (*err) st->timeout = 1;
}

}  // namespace

bool km_tc_supported(int d, int k) { return d == kKmD && k >= 1 && k <= kKmMaxK; }

int km_tc_create(fem_km *h) {
  KmTcPlanImpl *p = new (std::nothrow) KmTcPlanImpl();
  if (!p) return FEM_ERR_BAD_ARG;
  h->tc = p;
  p->kp = (h->k + 15) / 16 * 16;
  FEM_TRY(dalloc(&p->b1, (size_t)p->kp * 64));
  FEM_TRY(dalloc(&p->b2, (size_t)p->kp * 64));
  FEM_TRY(dalloc(&p->cconst, (size_t)3 * p->kp + 2));
  FEM_TRY(dalloc(&p->err, 1));
  FEM_CUDA(cudaMemset(p->err, 0, sizeof(int)));
  FEM_TRY(encode_tmap_2d(&p->tm_x, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->X, kKmD, (uint64_t)h->n, kKmD,
                         kKmTile, CU_TENSOR_MAP_SWIZZLE_128B));
  FEM_TRY(encode_tmap_2d(&p->tm_b1, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->b1, 64, (uint64_t)p->kp, 64, p->kp,
                         CU_TENSOR_MAP_SWIZZLE_128B));
  FEM_TRY(encode_tmap_2d(&p->tm_b2, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, p->b2, 64, (uint64_t)p->kp, 64, p->kp,
                         CU_TENSOR_MAP_SWIZZLE_128B));
  FEM_CUDA(cudaFuncSetAttribute(k_km_assign_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(KmSmem) + 1024)));
  return FEM_OK;
}

void km_tc_destroy(fem_km *h) {
  KmTcPlanImpl *p = static_cast<KmTcPlanImpl *>(h->tc);
  if (!p) return;
  dfree(p->b1);
  dfree(p->b2);
  dfree(p->cconst);
  dfree(p->err);
  delete p;
  h->tc = nullptr;
}

int km_tc_assign(fem_km *h) {
  KmTcPlanImpl *p = static_cast<KmTcPlanImpl *>(h->tc);
  FEM_CUDA(cudaMemsetAsync(p->cconst + 3 * p->kp, 0, 2 * sizeof(float), h->stream));
  k_km_tc_prep<<<p->kp, 64, 0, h->stream>>>(h->cent, h->g, h->k, p->kp, p->b1, p->b2, p->cconst);
  FEM_CUDA(cudaGetLastError());
  k_km_assign_tc<<<h->grid, kKmThreads, sizeof(KmSmem) + 1024, h->stream>>>(
      p->tm_x, p->tm_b1, p->tm_b2, p->cconst, h->cent, h->centf, h->cnorm, h->g, h->n, h->k, p->kp, h->labels, h->acc, h->cnt,
      ldexpf(1.f, h->shift), h->dstat, p->err);
  FEM_CUDA(cudaGetLastError());
  k_km_tc_flag<<<1, 1, 0, h->stream>>>(h->dstat, p->err);
  FEM_CUDA(cudaGetLastError());
  return FEM_OK;
}

}  // namespace fem
