// fem_oracle_blas.cpp -- the oracle's EM sweep with level-3 BLAS, for timing.
//
// TEST INFRASTRUCTURE ONLY (see fem_oracle.h).  Same arithmetic as
// orc_em_train's sweep, organised like the reference's SimpleMatrixEM: row
// blocks spread over OpenMP threads, each thread calling single-threaded BLAS
// (the reference calls MKL from inside its OpenMP regions):
//
//   factor  NormalDensity::Init (EM2/NormalDensity.cpp:43-65): Cholesky of
//           sym(lower(Sigma)), log det, U = (L^-1)^T upper
//   E-step  MatrixEMBase::BlockDensities (EM2/MatrixEM.cpp:69-81): T = X_blk -
//           mu_j, T <- T U_j (dtrmm), l = -1/2 rowsum(T^2) + c_j; then
//           PostProcessDensityMatrix (:39-51): log-sum-exp, posteriors, logL
//   M-step  SimpleMatrixEM::doMStep (:319-375): posterior sums, R^T X (dgemm),
//           mu = sums / N; T_j = (X - mu_j) sqrt(r_j), T_j^T T_j (dsyrk),
//           Sigma_j = sum / N_j; pi = N / n
//
// The BLAS entry points are passed in by the caller (CBLAS signatures), so the
// library links no BLAS itself.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <omp.h>

#include "fem_oracle.h"

namespace {

constexpr int kRowMajor = 101, kNoTrans = 111, kTrans = 112, kUpper = 121, kRight = 142, kNonUnit = 131;

typedef void (*dtrmm_t)(int, int, int, int, int, int, int, double, const double *, int, double *, int);
typedef void (*dgemm_t)(int, int, int, int, int, int, double, const double *, int, const double *, int, double,
                        double *, int);
typedef void (*dsyrk_t)(int, int, int, int, int, double, const double *, int, double, double *, int);

constexpr int kBlock = 256;

}  // namespace

// `sweeps` sweeps in one call, the way EMAlgorithm::TrainNoCopy
// (EM2/EMAlgorithm.cpp:139-191) runs them over buffers sized once (the
// posteriors N x K, the per-thread partials): factor, E-step with logL,
// M-step, and with `svd` the largest condition number of the new covariances
// (EMAlgorithm::FindLargestConditionNumber, EM2/EMAlgorithm.cpp:193-202; one
// eigen-solve per component, spread over the threads), stopping with
// ORC_ERR_COND_ABORT above `abort_thr`; parameters updated in place.
// logl[s] = the pre-M-step logL of sweep s, seconds[s] = its wall-clock time
// (omp_get_wtime), both may be null.
extern "C" int orc_em_sweeps_blas(int d, int64_t n, int k, const float *X, double *pi, double *mu, double *sigma,
                                  int sweeps, int svd, double abort_thr, double *logl, double *seconds,
                                  int nthreads, void *dtrmm_p, void *dgemm_p, void *dsyrk_p) {
  if (d < 1 || n < 1 || k < 1 || sweeps < 1 || !X || !pi || !mu || !sigma || !dtrmm_p || !dgemm_p || !dsyrk_p)
    return ORC_ERR_BAD_ARG;
  const dtrmm_t dtrmm = (dtrmm_t)dtrmm_p;
  const dgemm_t dgemm = (dgemm_t)dgemm_p;
  const dsyrk_t dsyrk = (dsyrk_t)dsyrk_p;
  const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
  const size_t dd = (size_t)d * d;
  const int64_t nblk = (n + kBlock - 1) / kBlock;

  std::vector<double> U(dd * k), c(k);
  std::vector<double> R((size_t)n * k);
  std::vector<double> part(nblk, 0.0);
  std::vector<double> N1((size_t)nt * k), S2((size_t)nt * k * d), Nj(k), C((size_t)nt * k * dd);

  for (int sw = 0; sw < sweeps; sw++) {
    const double t0 = omp_get_wtime();
    // ---- factor
    for (int j = 0; j < k; j++) {
      std::vector<double> L(dd, 0.0), Li(dd, 0.0);
      const double *S = sigma + dd * j;
      double ld = 0.0;
      for (int col = 0; col < d; col++) {
        double s = S[(size_t)col * d + col];
        for (int m = 0; m < col; m++) s -= L[(size_t)col * d + m] * L[(size_t)col * d + m];
        if (!(s > 0.0)) return ORC_ERR_CHOLESKY;
        const double l = std::sqrt(s);
        L[(size_t)col * d + col] = l;
        ld += std::log(l);
        for (int r = col + 1; r < d; r++) {
          double t = S[(size_t)r * d + col];
          for (int m = 0; m < col; m++) t -= L[(size_t)r * d + m] * L[(size_t)col * d + m];
          L[(size_t)r * d + col] = t / l;
        }
      }
      for (int col = 0; col < d; col++)
        for (int r = col; r < d; r++) {
          double s = (r == col) ? 1.0 : 0.0;
          for (int m = col; m < r; m++) s -= L[(size_t)r * d + m] * Li[(size_t)m * d + col];
          Li[(size_t)r * d + col] = s / L[(size_t)r * d + r];
        }
      for (int r = 0; r < d; r++)
        for (int col = 0; col < d; col++) U[dd * j + (size_t)r * d + col] = Li[(size_t)col * d + r];
      c[j] = std::log(pi[j]) - 0.5 * d * std::log(2.0 * M_PI) - ld;
    }

    // ---- E-step
#pragma omp parallel num_threads(nt)
    {
      std::vector<double> Xd((size_t)kBlock * d), T((size_t)kBlock * d), l((size_t)kBlock * k);
#pragma omp for schedule(dynamic, 4)
      for (int64_t b = 0; b < nblk; b++) {
        const int64_t r0 = b * kBlock;
        const int rows = (int)std::min<int64_t>(kBlock, n - r0);
        for (size_t e = 0; e < (size_t)rows * d; e++) Xd[e] = (double)X[(size_t)r0 * d + e];
        for (int j = 0; j < k; j++) {
          for (int r = 0; r < rows; r++)
            for (int q = 0; q < d; q++) T[(size_t)r * d + q] = Xd[(size_t)r * d + q] - mu[(size_t)j * d + q];
          dtrmm(kRowMajor, kRight, kUpper, kNoTrans, kNonUnit, rows, d, 1.0, U.data() + dd * j, d, T.data(), d);
          for (int r = 0; r < rows; r++) {
            double s = 0.0;
            for (int q = 0; q < d; q++) s += T[(size_t)r * d + q] * T[(size_t)r * d + q];
            l[(size_t)r * k + j] = -0.5 * s + c[j];
          }
        }
        double lsum = 0.0;
        for (int r = 0; r < rows; r++) {
          double m = l[(size_t)r * k];
          for (int j = 1; j < k; j++) m = std::fmax(m, l[(size_t)r * k + j]);
          double s = 0.0;
          for (int j = 0; j < k; j++) s += std::exp(l[(size_t)r * k + j] - m);
          const double lse = m + std::log(s);
          lsum += lse;
          for (int j = 0; j < k; j++) R[(size_t)(r0 + r) * k + j] = std::exp(l[(size_t)r * k + j] - lse);
        }
        part[b] = lsum;
      }
    }
    double ll = 0.0;
    for (double v : part) ll += v;
    if (logl) logl[sw] = ll;

    // ---- M-step: posterior sums and R^T X
    std::fill(N1.begin(), N1.end(), 0.0);
    std::fill(S2.begin(), S2.end(), 0.0);
#pragma omp parallel num_threads(nt)
    {
      const int t = omp_get_thread_num();
      std::vector<double> Xd((size_t)kBlock * d);
#pragma omp for schedule(static)
      for (int64_t b = 0; b < nblk; b++) {
        const int64_t r0 = b * kBlock;
        const int rows = (int)std::min<int64_t>(kBlock, n - r0);
        for (size_t e = 0; e < (size_t)rows * d; e++) Xd[e] = (double)X[(size_t)r0 * d + e];
        for (int r = 0; r < rows; r++)
          for (int j = 0; j < k; j++) N1[(size_t)t * k + j] += R[(size_t)(r0 + r) * k + j];
        dgemm(kRowMajor, kTrans, kNoTrans, k, d, rows, 1.0, R.data() + (size_t)r0 * k, k, Xd.data(), d, 1.0,
              S2.data() + (size_t)t * k * d, d);
      }
    }
    for (int j = 0; j < k; j++) {
      Nj[j] = 0.0;
      for (int t = 0; t < nt; t++) Nj[j] += N1[(size_t)t * k + j];
      for (int q = 0; q < d; q++) {
        double s = 0.0;
        for (int t = 0; t < nt; t++) s += S2[((size_t)t * k + j) * d + q];
        mu[(size_t)j * d + q] = s / Nj[j];
      }
      pi[j] = Nj[j] / (double)n;
    }

    // ---- M-step: covariances around the new means
    std::fill(C.begin(), C.end(), 0.0);
#pragma omp parallel num_threads(nt)
    {
      const int t = omp_get_thread_num();
      std::vector<double> T((size_t)kBlock * d);
#pragma omp for schedule(static)
      for (int64_t b = 0; b < nblk; b++) {
        const int64_t r0 = b * kBlock;
        const int rows = (int)std::min<int64_t>(kBlock, n - r0);
        for (int j = 0; j < k; j++) {
          for (int r = 0; r < rows; r++) {
            const double w = std::sqrt(R[(size_t)(r0 + r) * k + j]);
            for (int q = 0; q < d; q++)
              T[(size_t)r * d + q] = ((double)X[(size_t)(r0 + r) * d + q] - mu[(size_t)j * d + q]) * w;
          }
          dsyrk(kRowMajor, kUpper, kTrans, d, rows, 1.0, T.data(), d, 1.0, C.data() + ((size_t)t * k + j) * dd,
                d);
        }
      }
    }
    for (int j = 0; j < k; j++)
      for (int a = 0; a < d; a++)
        for (int b2 = a; b2 < d; b2++) {
          double s = 0.0;
          for (int t = 0; t < nt; t++) s += C[((size_t)t * k + j) * dd + (size_t)a * d + b2];
          s /= Nj[j];
          sigma[dd * j + (size_t)a * d + b2] = s;
          sigma[dd * j + (size_t)b2 * d + a] = s;
        }
    double cond = 0.0;
    if (svd) {
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1) reduction(max : cond)
      for (int j = 0; j < k; j++) cond = std::max(cond, orc_cond_number(d, sigma + dd * j));
    }
    if (seconds) seconds[sw] = omp_get_wtime() - t0;
    if (svd && cond > abort_thr) return ORC_ERR_COND_ABORT;
  }
  return ORC_OK;
}

extern "C" int orc_em_sweep_blas(int d, int64_t n, int k, const float *X, double *pi, double *mu, double *sigma,
                                 double *logl, int nthreads, void *dtrmm_p, void *dgemm_p, void *dsyrk_p) {
  if (!logl) return ORC_ERR_BAD_ARG;
  return orc_em_sweeps_blas(d, n, k, X, pi, mu, sigma, 1, 0, 0.0, logl, nullptr, nthreads, dtrmm_p, dgemm_p,
                            dsyrk_p);
}
