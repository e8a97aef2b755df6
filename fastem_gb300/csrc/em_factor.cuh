// em_factor.cuh -- block-wide FP64 steps on one d x d covariance matrix,
// shared by the single-fit kernels (em_plain.cu) and the batched engine
// (em_batch.cu).  Every thread of the block calls each function; matrices are
// row-major d x d in global or shared memory.
#pragma once

#include <cmath>

namespace fem {

// EMAlgorithm::RegularizeCovariances (EM2/EMAlgorithm.cpp:237-244):
// S <- (1 - reg) S + (reg tr(S) / d) I, in place.
__device__ inline void block_regularize(double *S, int d, double reg) {
  __shared__ double s_add;
  if (threadIdx.x == 0) {
    double tr = 0.0;
    for (int q = 0; q < d; q++) tr += S[(size_t)q * d + q];
    s_add = reg * tr / (double)d;
  }
  __syncthreads();
  const double add = s_add;
  for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
    const int r = e / d, c = e - r * d;
    S[e] = S[e] * (1.0 - reg) + (r == c ? add : 0.0);
  }
  __syncthreads();
}

// NormalDensity::Init (EM2/NormalDensity.cpp:43-65): A <- sym(lower(S)),
// then right-looking Cholesky in place (L in the lower triangle).  A pivot
// <= 0 fails, as Eigen's LLT reports.  Returns true on success, the same in
// every thread.
__device__ inline bool block_cholesky(const double *S, int d, double *A) {
  __shared__ double s_piv;
  __shared__ int s_fail;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < d * d; e += nt) {
    const int r = e / d, c = e - r * d;
    A[e] = (c <= r) ? S[e] : S[(size_t)c * d + r];
  }
  if (tid == 0) s_fail = 0;
  __syncthreads();
  for (int k = 0; k < d; k++) {
    if (tid == 0) {
      const double x = A[(size_t)k * d + k];
      if (!(x > 0.0)) {
        s_fail = 1;
      } else {
        const double l = sqrt(x);
        A[(size_t)k * d + k] = l;
        s_piv = l;
      }
    }
    __syncthreads();
    if (s_fail) break;
    const double lkk = s_piv;
    for (int i = k + 1 + tid; i < d; i += nt) A[(size_t)i * d + k] /= lkk;
    __syncthreads();
    // trailing update of the lower triangle: A[i][c] -= L[i][k] L[c][k], k < c <= i
    const int m = d - k - 1;
    for (int e = tid; e < m * m; e += nt) {
      const int i = e / m, c = e - i * m;
      if (c > i) continue;
      const int gi = k + 1 + i, gc = k + 1 + c;
      A[(size_t)gi * d + gc] -= A[(size_t)gi * d + k] * A[(size_t)gc * d + k];
    }
    __syncthreads();
  }
  const bool ok = !s_fail;
  __syncthreads();
  return ok;
}

constexpr int kFactorMaxD = 256;   // largest d of the block factorisation helpers

// W = L^-1 (lower, row-major) by forward substitution, threads owning columns;
// L is the lower triangle of A.  The diagonal's reciprocals are formed once,
// in parallel, so a column's substitution multiplies instead of dividing.
// d <= kFactorMaxD.
__device__ inline void block_lower_inverse(const double *A, int d, double *Wi) {
  __shared__ double s_rd[kFactorMaxD];
  for (int r = threadIdx.x; r < d; r += blockDim.x) s_rd[r] = 1.0 / A[(size_t)r * d + r];
  __syncthreads();
  for (int c = threadIdx.x; c < d; c += blockDim.x) {
    for (int r = 0; r < c; r++) Wi[(size_t)r * d + c] = 0.0;
    for (int r = c; r < d; r++) {
      double s = (r == c) ? 1.0 : 0.0;
      for (int m2 = c; m2 < r; m2++) s -= A[(size_t)r * d + m2] * Wi[(size_t)m2 * d + c];
      Wi[(size_t)r * d + c] = s * s_rd[r];
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------------
// Blocked forms of block_cholesky and block_lower_inverse for one CTA of
// kFactorThreads threads (d <= kFactorMaxD).  Each matrix element goes through
// the same FP64 operations in the same order as in the unblocked functions (a
// running a - x y per update, k ascending), so the factors are bit-identical;
// the blocking only changes where the operands live.  With one CTA per
// component the unblocked loops wait on L2 for every element update; here the
// panel being factored and the row block being inverted sit in shared memory,
// the trailing updates are 4 x 4 register tiles, and the FP64 pipe is the
// limit (d^3 / 6 fused multiply-adds each for the factor and the inverse).
constexpr int kFactorThreads = 256;
constexpr int kPanel = 32;                // columns per Cholesky panel, rows per inverse block
constexpr int kPanelLd = kPanel + 1;      // panel row stride (doubles)
constexpr int kFactorBlockedD = 128;      // smallest d that the blocked forms are used for

// dynamic shared memory of the two functions (the panel, then the row block)
__host__ __device__ constexpr size_t factor_smem_bytes(int d) {
  return (size_t)d * kPanelLd * sizeof(double);
}

// block_cholesky with panels of kPanel columns: the panel (rows k0 .. d-1)
// is factored in shared memory (thread i owns row k0 + i), written back, and
// its update of the trailing lower triangle applied as 4 x 4 tiles.  The
// upper triangle of A keeps the symmetric copy of S, as in block_cholesky.
// P: factor_smem_bytes(d) of shared memory.  Returns true on success, the
// same in every thread.
__device__ inline bool block_cholesky_panels(const double *S, int d, double *A, double *P) {
  __shared__ double s_diag[kPanel];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < d * d; e += nt) {
    const int r = e / d, c = e - r * d;
    A[e] = (c <= r) ? S[e] : S[(size_t)c * d + r];
  }
  __syncthreads();
  bool ok = true;
  for (int k0 = 0; k0 < d; k0 += kPanel) {
    const int w = min(kPanel, d - k0), m = d - k0;
    for (int e = tid; e < m * w; e += nt) {
      const int i = e / w, q = e - i * w;
      P[i * kPanelLd + q] = A[(size_t)(k0 + i) * d + k0 + q];
    }
    __syncthreads();
    const int i = tid;                    // panel row owned by this thread
    for (int q = 0; q < w; q++) {
      const double x = P[q * kPanelLd + q];   // the same value in every thread
      if (!(x > 0.0)) {
        ok = false;
        break;
      }
      const double l = sqrt(x);
      if (i == q) s_diag[q] = l;
      if (i > q && i < m) P[i * kPanelLd + q] = P[i * kPanelLd + q] / l;
      __syncthreads();
      if (i > q && i < m) {
        const double lik = P[i * kPanelLd + q];
        const int ce = min(i, w - 1);
        for (int c = q + 1; c <= ce; c++)
          P[i * kPanelLd + c] = fma(-lik, P[c * kPanelLd + q], P[i * kPanelLd + c]);
      }
      __syncthreads();
    }
    if (!ok) break;
    for (int e = tid; e < m * w; e += nt) {
      const int r = e / w, q = e - r * w;
      if (q <= r) A[(size_t)(k0 + r) * d + k0 + q] = (q == r) ? s_diag[q] : P[r * kPanelLd + q];
    }
    // trailing update: A[r][c] -= sum_q L[r][q] L[c][q], w <= c <= r < m
    // (panel-relative), over 4 x 4 tiles of the lower triangle
    const int n2 = m - w;
    if (n2 > 0) {
      const int T = (n2 + 3) >> 2;
      const int ntile = T * (T + 1) / 2;
      for (int t = tid; t < ntile; t += nt) {
        int ti = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
        while ((ti + 1) * (ti + 2) / 2 <= t) ti++;
        while (ti * (ti + 1) / 2 > t) ti--;
        const int tc = t - ti * (ti + 1) / 2;
        const int rb = w + 4 * ti, cb = w + 4 * tc;
        double acc[4][4];
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
          for (int v = 0; v < 4; v++) {
            const int r = rb + u, c = cb + v;
            acc[u][v] = (r < m && c <= r) ? A[(size_t)(k0 + r) * d + k0 + c] : 0.0;
          }
        for (int q = 0; q < w; q++) {
          double a[4], b[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            a[u] = (rb + u < m) ? P[(rb + u) * kPanelLd + q] : 0.0;
            b[u] = (cb + u < m) ? P[(cb + u) * kPanelLd + q] : 0.0;
          }
#pragma unroll
          for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] = fma(-a[u], b[v], acc[u][v]);
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
          for (int v = 0; v < 4; v++) {
            const int r = rb + u, c = cb + v;
            if (r < m && c <= r) A[(size_t)(k0 + r) * d + k0 + c] = acc[u][v];
          }
      }
    }
    __syncthreads();
  }
  __syncthreads();
  return ok;
}

// block_lower_inverse by blocks of kPanel rows, thread c owning column c of
// W = L^-1 (d <= blockDim.x): the block's rows of L are staged in shared
// memory (Lb); the terms of the rows above the block (m < r0) run as a
// register-blocked product over the thread's own column of W, then the
// block's triangle is solved row by row with that column's new entries in
// registers.  Terms with m < c multiply an exact zero of W and leave the
// running sum unchanged, so the loops need no per-column bounds.
__device__ inline void block_lower_inverse_rows(const double *A, int d, double *Wi, double *Lb) {
  __shared__ double s_rd[kFactorMaxD];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int r = tid; r < d; r += nt) s_rd[r] = 1.0 / A[(size_t)r * d + r];
  const int c = tid;
  for (int r0 = 0; r0 < d; r0 += kPanel) {
    const int rb = min(kPanel, d - r0), mw = r0 + rb;   // block rows, columns of L used
    __syncthreads();                                    // Lb free (and s_rd formed)
    for (int e = tid; e < kPanel * mw; e += nt) {
      const int rr = e / mw, m = e - rr * mw;
      Lb[rr * mw + m] = rr < rb ? A[(size_t)(r0 + rr) * d + m] : 0.0;
    }
    __syncthreads();
    if (c >= d) continue;
    if (c >= mw) {                                      // above the diagonal
      for (int rr = 0; rr < rb; rr++) Wi[(size_t)(r0 + rr) * d + c] = 0.0;
      continue;
    }
    double acc[kPanel];
#pragma unroll
    for (int rr = 0; rr < kPanel; rr++) acc[rr] = 0.0;
    for (int m = c; m < r0; m++) {                      // rows above the block
      const double wm = Wi[(size_t)m * d + c];
#pragma unroll
      for (int rr = 0; rr < kPanel; rr++) acc[rr] = fma(-Lb[rr * mw + m], wm, acc[rr]);
    }
    double wb[kPanel];
#pragma unroll
    for (int rr = 0; rr < kPanel; rr++) {               // the block's triangle
      if (rr < rb) {
        const int r = r0 + rr;
        double s = c < r0 ? acc[rr] : (r == c ? 1.0 : 0.0);
#pragma unroll
        for (int mm = 0; mm < rr; mm++) s = fma(-Lb[rr * mw + r0 + mm], wb[mm], s);
        wb[rr] = r < c ? 0.0 : s * s_rd[r];
        Wi[(size_t)r * d + c] = wb[rr];
      }
    }
  }
  __syncthreads();
}

// log det = 2 sum log L_ii (L in the lower triangle of A): the logarithms in
// parallel, summed in index order by one thread; the value in every thread.
// d <= kFactorMaxD.
__device__ inline double block_chol_logdet(const double *A, int d) {
  __shared__ double s_log[kFactorMaxD];
  __shared__ double s_ld;
  for (int q = threadIdx.x; q < d; q += blockDim.x) s_log[q] = log(A[(size_t)q * d + q]);
  __syncthreads();
  if (threadIdx.x == 0) {
    double ld = 0.0;
    for (int q = 0; q < d; q++) ld += s_log[q];
    s_ld = 2.0 * ld;
  }
  __syncthreads();
  const double v = s_ld;
  __syncthreads();
  return v;
}

// An upper bound of the condition number lambda_max / lambda_min of the
// positive definite sym(lower(S)) = L L^T, from norms only:
//   lambda_max <= ||Sigma||_F and 1 / lambda_min = ||L^-1||_2^2 <= ||L^-1||_F^2.
// S is row-major (its lower triangle is used), Wi = L^-1 (lower).  At most
// d^1.5 times the true value; the caller runs the exact eigenvalues
// (block_jacobi_cond) only when the bound does not settle a test.  Sums in a
// fixed order; the value in every thread.  blockDim.x <= 256.
__device__ inline double block_cond_bound(const double *S, const double *Wi, int d) {
  __shared__ double red_s[256], red_w[256];
  __shared__ double s_b;
  const int tid = threadIdx.x, nt = blockDim.x;
  double fs = 0.0, fw = 0.0;
  for (int e = tid; e < d * d; e += nt) {
    const int r = e / d, c = e - r * d;
    if (c > r) continue;
    const double v = S[e], w = Wi[e];
    fs += (c == r ? 1.0 : 2.0) * v * v;
    fw += w * w;
  }
  red_s[tid] = fs;
  red_w[tid] = fw;
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, b = 0.0;
    for (int t = 0; t < nt; t++) a += red_s[t], b += red_w[t];
    s_b = sqrt(a) * b;
  }
  __syncthreads();
  const double v = s_b;
  __syncthreads();
  return v;
}

// NormalDensity::ComputeConditionNumber (EM2/NormalDensity.cpp:67-71): the
// eigenvalues of the symmetric matrix in A (overwritten) by cyclic Jacobi in
// FP64.  Each sweep runs the n - 1 rounds of a round-robin schedule; a round
// rotates n / 2 disjoint (p, q) pairs at once (columns, then rows).  Sweeps
// stop when the off-diagonal mass is below 1e-30 of the diagonal's, or after
// 100.  Returns |max eig / min eig| in every thread.  blockDim.x <= 256,
// d <= 256.
__device__ inline double block_jacobi_cond(double *A, int d) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int n = d + (d & 1);          // players of the round robin (a dummy when d is odd)
  const int np = n / 2;
  __shared__ double sc[128], ss[128];
  __shared__ int sp[128], sq[128];
  __shared__ double red_off[256], red_diag[256];
  __shared__ int done;
  __shared__ double s_cond;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, dg = 0.0;
    for (int e = tid; e < d * d; e += nt) {
      const int r = e / d, c = e - r * d;
      const double v = A[e];
      if (c > r) off += v * v;
      else if (c == r) dg += v * v;
    }
    red_off[tid] = off;
    red_diag[tid] = dg;
    __syncthreads();
    if (tid == 0) {
      double o = 0.0, g = 0.0;
      for (int t = 0; t < nt; t++) o += red_off[t], g += red_diag[t];
      done = !(o > 1e-30 * g);
    }
    __syncthreads();
    if (done) break;
    for (int round = 0; round < n - 1; round++) {
      for (int i = tid; i < np; i += nt) {
        // position m holds player 0 (m = 0) or 1 + (m - 1 + round) mod (n - 1)
        const int m1 = i, m2 = n - 1 - i;
        const int p0 = m1 == 0 ? 0 : 1 + (m1 - 1 + round) % (n - 1);
        const int q0 = 1 + (m2 - 1 + round) % (n - 1);
        const int p = min(p0, q0), q = max(p0, q0);
        double c = 1.0, s = 0.0;
        if (q < d) {
          const double apq = A[(size_t)p * d + q];
          if (apq != 0.0) {
            const double app = A[(size_t)p * d + p], aqq = A[(size_t)q * d + q];
            const double th = (aqq - app) / (2.0 * apq);
            const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            s = t * c;
          }
        }
        sc[i] = c, ss[i] = s, sp[i] = p, sq[i] = q;
      }
      __syncthreads();
      for (int e = tid; e < d * np; e += nt) {     // columns p, q of every row
        const int i = e / d, r = e - i * d;
        const int p = sp[i], q = sq[i];
        if (q < d && ss[i] != 0.0) {
          const double arp = A[(size_t)r * d + p], arq = A[(size_t)r * d + q];
          A[(size_t)r * d + p] = sc[i] * arp - ss[i] * arq;
          A[(size_t)r * d + q] = ss[i] * arp + sc[i] * arq;
        }
      }
      __syncthreads();
      for (int e = tid; e < d * np; e += nt) {     // rows p, q of every column
        const int i = e / d, r = e - i * d;
        const int p = sp[i], q = sq[i];
        if (q < d && ss[i] != 0.0) {
          const double apr = A[(size_t)p * d + r], aqr = A[(size_t)q * d + r];
          A[(size_t)p * d + r] = sc[i] * apr - ss[i] * aqr;
          A[(size_t)q * d + r] = ss[i] * apr + sc[i] * aqr;
        }
      }
      __syncthreads();
    }
  }
  if (tid == 0) {
    double mn = A[0], mx = A[0];
    for (int p = 1; p < d; p++) {
      mn = fmin(mn, A[(size_t)p * d + p]);
      mx = fmax(mx, A[(size_t)p * d + p]);
    }
    s_cond = fabs(mx / mn);
  }
  __syncthreads();
  const double cond = s_cond;
  __syncthreads();
  return cond;
}

}  // namespace fem
