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
