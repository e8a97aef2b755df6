/*
 * fem_oracle.cpp -- FP64 CPU restatement of FastEM's EM (SimpleMatrixEM) and
 * k-means (NaiveKMA) hot path, plus the host-side seeders the benchmark
 * configurations start from.
 *
 * TEST INFRASTRUCTURE ONLY (see fem_oracle.h): the checker and the timed CPU
 * baseline, never part of the shipped library.  PARITY UNPINNED for the EM
 * and k-means arithmetic: the reference cannot be built here and has no
 * golden vectors; this code is cross-checked against an independent
 * numpy/scipy FP64 computation.  The generator stream (orc_rng_*) is pinned:
 * it equals the reference's own Util/Rand.cpp, compiled in place by
 * `make ref` (Makefile), bit for bit.
 *
 * Arithmetic notes.  Everything is IEEE double with sequential summation in
 * index order; the file is compiled with -ffp-contract=off so x86 and Arm
 * builds give identical bits.  The reference's OpenMP reductions sum partial
 * results in an unspecified order; here per-thread partials are combined in
 * thread order (deterministic for a given thread count).
 */
#include "fem_oracle.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

namespace {

/* Util/Rand.cpp:7-36: one global engine and distribution. */
std::mt19937_64 g_rng;
std::uniform_real_distribution<> g_uniform;

int resolve_threads(int nthreads) {
  return nthreads > 0 ? nthreads : omp_get_max_threads();
}

/* Util/OpenMP.h:37-47 FindOpenMPItems: contiguous split of nItems rows. */
void find_items(int64_t n, int size, int id, int64_t &off, int64_t &cnt) {
  cnt = n / size;
  int64_t rem = n % size;
  if (id < rem) {
    cnt++;
    off = cnt * id;
  } else {
    off = cnt * id + rem;
  }
}

/* Eigen LLT unblocked criterion (pivot <= 0 fails); lower factor in L. */
bool cholesky_lower(int d, const double *C, double *L) {
  for (int i = 0; i < d * d; i++) L[i] = 0.0;
  for (int k = 0; k < d; k++) {
    double x = C[k * d + k];
    for (int m = 0; m < k; m++) x -= L[k * d + m] * L[k * d + m];
    if (!(x > 0.0)) return false;
    double lkk = std::sqrt(x);
    L[k * d + k] = lkk;
    for (int i = k + 1; i < d; i++) {
      double s = C[i * d + k];
      for (int m = 0; m < k; m++) s -= L[i * d + m] * L[k * d + m];
      L[i * d + k] = s / lkk;
    }
  }
  return true;
}

/* L X = I by forward substitution; returns U = X^T (upper). */
void inverse_transpose(int d, const double *L, double *U) {
  std::vector<double> X(d * d, 0.0);
  for (int c = 0; c < d; c++) {
    for (int r = c; r < d; r++) {
      double s = (r == c) ? 1.0 : 0.0;
      for (int m = c; m < r; m++) s -= L[r * d + m] * X[m * d + c];
      X[r * d + c] = s / L[r * d + r];
    }
  }
  for (int r = 0; r < d; r++)
    for (int c = 0; c < d; c++) U[r * d + c] = X[c * d + r];
}

/* symmetric copy from the lower triangle (selfadjointView<Lower>) */
void sym_from_lower(int d, const double *S, double *C) {
  for (int r = 0; r < d; r++)
    for (int c = 0; c < d; c++)
      C[r * d + c] = (c <= r) ? S[r * d + c] : S[c * d + r];
}

/* cyclic Jacobi eigenvalues of a symmetric matrix (destroys A) */
void jacobi_eigenvalues(int d, double *A, double *ev) {
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int p = 0; p < d; p++) {
      diag += A[p * d + p] * A[p * d + p];
      for (int q = p + 1; q < d; q++) off += A[p * d + q] * A[p * d + q];
    }
    if (off <= 1e-30 * diag) break;
    for (int p = 0; p < d; p++) {
      for (int q = p + 1; q < d; q++) {
        double apq = A[p * d + q];
        if (apq == 0.0) continue;
        double app = A[p * d + p], aqq = A[q * d + q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) /
                   (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int r = 0; r < d; r++) {
          double arp = A[r * d + p], arq = A[r * d + q];
          A[r * d + p] = c * arp - s * arq;
          A[r * d + q] = s * arp + c * arq;
        }
        for (int r = 0; r < d; r++) {
          double apr = A[p * d + r], aqr = A[q * d + r];
          A[p * d + r] = c * apr - s * aqr;
          A[q * d + r] = s * apr + c * aqr;
        }
      }
    }
  }
  for (int p = 0; p < d; p++) ev[p] = A[p * d + p];
}

/* CentroidVector::SquaredDistance(int k, vec, row) (Clust/CentroidVector.h:90-102):
 * centroid in double, row converted to double, sequential sum over columns. */
inline double sqdist_dd(int d, const double *c, const double *x) {
  double s = 0.0;
  for (int q = 0; q < d; q++) {
    double t = c[q] - x[q];
    s += t * t;
  }
  return s;
}

/* CentroidVector::SquaredDistance(const float*, const float*)
 * (Clust/CentroidVector.h:79-88): differences and squares in float,
 * accumulated in double. */
inline double sqdist_ff(int d, const float *a, const float *b) {
  double s = 0.0;
  for (int q = 0; q < d; q++) {
    float t = b[q] - a[q];
    float t2 = t * t;
    s += (double)t2;
  }
  return s;
}

/* CentroidVector::SquaredDistance(int k, vec, const float* row)
 * (Clust/CentroidVector.h:104-116): double centroid minus float row. */
inline double sqdist_df(int d, const double *c, const float *x) {
  double s = 0.0;
  for (int q = 0; q < d; q++) {
    double t = c[q] - (double)x[q];
    s += t * t;
  }
  return s;
}

}  // namespace

extern "C" {

void orc_rng_seed(uint64_t seed) {
  /* SRand takes an unsigned (Util/Rand.cpp:33-35) */
  g_rng.seed((unsigned)seed);
  g_uniform.reset();
}

double orc_rng_uniform(void) { return g_uniform(g_rng); }

/* ------------------------------------------------------------------ EM */

int orc_em_init_densities(int d, int k, const double *sigma, double *U,
                          double *logdet, int *failed) {
  if (failed) *failed = -1;
  std::vector<double> C(d * d), L(d * d);
  for (int j = 0; j < k; j++) {
    sym_from_lower(d, sigma + (size_t)j * d * d, C.data());
    if (!cholesky_lower(d, C.data(), L.data())) {
      if (failed) *failed = j;
      return ORC_ERR_CHOLESKY;
    }
    double ld = 0.0;
    for (int q = 0; q < d; q++) ld += std::log(L[q * d + q]);
    logdet[j] = 2.0 * ld;
    inverse_transpose(d, L.data(), U + (size_t)j * d * d);
  }
  return ORC_OK;
}

void orc_em_regularize(int d, int k, double reg_coef, double *sigma) {
  for (int j = 0; j < k; j++) {
    double *S = sigma + (size_t)j * d * d;
    double tr = 0.0;
    for (int q = 0; q < d; q++) tr += S[q * d + q];
    double add = reg_coef * tr / (double)d;
    for (int r = 0; r < d; r++)
      for (int c = 0; c < d; c++)
        S[r * d + c] = S[r * d + c] * (1.0 - reg_coef) + (r == c ? add : 0.0);
  }
}

double orc_cond_number(int d, const double *sigma) {
  std::vector<double> A(d * d), ev(d);
  sym_from_lower(d, sigma, A.data());
  jacobi_eigenvalues(d, A.data(), ev.data());
  double mn = ev[0], mx = ev[0];
  for (int q = 1; q < d; q++) {
    mn = std::min(mn, ev[q]);
    mx = std::max(mx, ev[q]);
  }
  return std::fabs(mx / mn);
}

int orc_em_estep(int d, int64_t n, int k, const float *X, const double *pi,
                 const double *mu, const double *U, const double *logdet,
                 double *post, double *logl, int nthreads) {
  nthreads = resolve_threads(nthreads);
  /* MatrixEMBase::CalcLogCoeffs (EM2/MatrixEM.cpp:83-87) */
  std::vector<double> coef(k);
  const double logc = -0.5 * d * std::log(2.0 * M_PI);
  for (int j = 0; j < k; j++) coef[j] = std::log(pi[j]) + logc - 0.5 * logdet[j];

  std::vector<double> part(nthreads, 0.0);
  const int64_t BLK = 256;
#pragma omp parallel num_threads(nthreads)
  {
    int tid = omp_get_thread_num();
    int64_t off, cnt;
    find_items(n, nthreads, tid, off, cnt);
    std::vector<double> lw(BLK * k), t(d), y(d);
    double tl = 0.0;
    for (int64_t b0 = off; b0 < off + cnt; b0 += BLK) {
      int64_t bn = std::min(BLK, off + cnt - b0);
      /* BlockDensities: per component, rowwise subtract, TRMM, square-sum */
      for (int j = 0; j < k; j++) {
        const double *Uj = U + (size_t)j * d * d;
        const double *mj = mu + (size_t)j * d;
        for (int64_t i = 0; i < bn; i++) {
          const float *x = X + (b0 + i) * d;
          for (int q = 0; q < d; q++) {
            t[q] = (double)x[q] - mj[q];
            y[q] = 0.0;
          }
          /* T := T * U, U upper (cblas_dtrmm Right/Upper/NoTrans) */
          for (int m = 0; m < d; m++) {
            double tm = t[m];
            const double *Um = Uj + (size_t)m * d;
            for (int q = m; q < d; q++) y[q] += tm * Um[q];
          }
          double s = 0.0;
          for (int q = 0; q < d; q++) s += y[q] * y[q];
          lw[i * k + j] = -0.5 * s + coef[j];
        }
      }
      /* PostProcessDensityMatrix */
      for (int64_t i = 0; i < bn; i++) {
        const double *row = &lw[i * k];
        double mx = row[0];
        for (int j = 1; j < k; j++) mx = std::max(mx, row[j]);
        double se = 0.0;
        for (int j = 0; j < k; j++) se += std::exp(row[j] - mx);
        double lse = std::log(se) + mx;
        tl += lse;
        double *pr = post + (b0 + i) * k;
        for (int j = 0; j < k; j++) pr[j] = std::exp(row[j] - lse);
      }
    }
    part[tid] = tl;
  }
  double s = 0.0;
  for (int t = 0; t < nthreads; t++) s += part[t];
  *logl = s;
  return ORC_OK;
}

/* PosteriorSum and MeanSums per thread, reduced into thread 0's in thread
 * order, mu = MeanSums / PosteriorSum: the same in SimpleMatrixEM::doMStep
 * (EM2/MatrixEM.cpp:319-343) and CachedEM::ComputeMeansPostSum
 * (EM2/CachedEM.cpp:88-118).  ps receives the posterior sums. */
static void mstep_means(int d, int64_t n, int k, const float *X, const double *post, double *mu,
                        std::vector<double> &ps, int nthreads) {
  const size_t kd = (size_t)k * d;
  /* Step1ReducerData per thread: PosteriorSum[K], MeanSums[K x d] */
  ps.assign((size_t)nthreads * k, 0.0);
  std::vector<double> ms((size_t)nthreads * kd, 0.0);
#pragma omp parallel num_threads(nthreads)
  {
    int tid = omp_get_thread_num();
    int64_t off, cnt;
    find_items(n, nthreads, tid, off, cnt);
    double *tps = &ps[(size_t)tid * k];
    double *tms = &ms[(size_t)tid * kd];
    for (int64_t i = off; i < off + cnt; i++) {
      const double *r = post + i * k;
      const float *x = X + i * d;
      for (int j = 0; j < k; j++) {
        double rj = r[j];
        tps[j] += rj;
        double *mj = tms + (size_t)j * d;
        for (int q = 0; q < d; q++) mj[q] += rj * (double)x[q];
      }
    }
  }
  /* NaiveOMPReducer::ReduceToFirstThread (Util/OMPReducer.h:40-56) */
  for (int t = 1; t < nthreads; t++) {
    for (int j = 0; j < k; j++) ps[j] += ps[(size_t)t * k + j];
    for (size_t q = 0; q < kd; q++) ms[q] += ms[(size_t)t * kd + q];
  }
  for (int j = 0; j < k; j++)
    for (int q = 0; q < d; q++) mu[(size_t)j * d + q] = ms[(size_t)j * d + q] / ps[j];
}

int orc_em_mstep_cached(int d, int64_t n, int k, const float *X, const double *post,
                        double *pi, double *mu, double *sigma, int nthreads) {
  nthreads = resolve_threads(nthreads);
  const size_t kdd = (size_t)k * d * d;
  std::vector<double> ps;
  mstep_means(d, n, k, X, post, mu, ps, nthreads);
  /* CachedEM::ComputeCovariances (EM2/CachedEM.cpp:120-163): per thread and
   * component, syr-style rank-1 updates of the upper triangle weighted by the
   * unscaled posterior around the new means; after the reduction the sums
   * are divided by the posterior sum (selfadjointView<Upper>). */
  std::vector<double> cs((size_t)nthreads * kdd, 0.0);
#pragma omp parallel num_threads(nthreads)
  {
    int tid = omp_get_thread_num();
    int64_t off, cnt;
    find_items(n, nthreads, tid, off, cnt);
    std::vector<double> t(d);
    for (int j = 0; j < k; j++) {
      double *C = &cs[(size_t)tid * kdd + (size_t)j * d * d];
      const double *mj = mu + (size_t)j * d;
      for (int64_t i = off; i < off + cnt; i++) {
        const double w = post[i * k + j];
        const float *x = X + i * d;
        for (int q = 0; q < d; q++) t[q] = (double)x[q] - mj[q];
        for (int a = 0; a < d; a++) {
          const double ta = w * t[a];
          double *Ca = C + (size_t)a * d;
          for (int b = a; b < d; b++) Ca[b] += ta * t[b];
        }
      }
    }
  }
  for (int t = 1; t < nthreads; t++)
    for (size_t q = 0; q < kdd; q++) cs[q] += cs[(size_t)t * kdd + q];
  for (int j = 0; j < k; j++) {
    const double *C = &cs[(size_t)j * d * d];
    double *S = sigma + (size_t)j * d * d;
    const double inv = 1.0 / ps[j];
    for (int a = 0; a < d; a++)
      for (int b = 0; b < d; b++) S[a * d + b] = inv * ((b >= a) ? C[a * d + b] : C[b * d + a]);
    /* CachedEM::MStep (EM2/CachedEM.cpp:166-170): Probs /= TotalRowCount */
    pi[j] = ps[j] / (double)n;
  }
  return ORC_OK;
}

int orc_em_mstep(int d, int64_t n, int k, const float *X, const double *post,
                 double *pi, double *mu, double *sigma, int nthreads) {
  nthreads = resolve_threads(nthreads);
  const size_t kdd = (size_t)k * d * d;
  std::vector<double> ps;
  mstep_means(d, n, k, X, post, mu, ps, nthreads);

  /* Step2ReducerData per thread: CovSums[K][d x d] (upper filled) */
  std::vector<double> cs((size_t)nthreads * kdd, 0.0);
#pragma omp parallel num_threads(nthreads)
  {
    int tid = omp_get_thread_num();
    int64_t off, cnt;
    find_items(n, nthreads, tid, off, cnt);
    std::vector<double> t(d);
    for (int j = 0; j < k; j++) {
      double *C = &cs[(size_t)tid * kdd + (size_t)j * d * d];
      const double *mj = mu + (size_t)j * d;
      /* ComputeWeightedTempDataset (EM2/MatrixEM.cpp:53-67) */
      double inv_sqrt_ps = 1.0 / std::sqrt(ps[j]);
      for (int64_t i = off; i < off + cnt; i++) {
        double sp = std::sqrt(post[i * k + j]) * inv_sqrt_ps;
        const float *x = X + i * d;
        for (int q = 0; q < d; q++) t[q] = ((double)x[q] - mj[q]) * sp;
        /* selfadjointView<Upper>().rankUpdate */
        for (int a = 0; a < d; a++) {
          double ta = t[a];
          double *Ca = C + (size_t)a * d;
          for (int b = a; b < d; b++) Ca[b] += ta * t[b];
        }
      }
    }
  }
  for (int t = 1; t < nthreads; t++)
    for (size_t q = 0; q < kdd; q++) cs[q] += cs[(size_t)t * kdd + q];
  for (int j = 0; j < k; j++) {
    const double *C = &cs[(size_t)j * d * d];
    double *S = sigma + (size_t)j * d * d;
    for (int a = 0; a < d; a++)
      for (int b = 0; b < d; b++) S[a * d + b] = (b >= a) ? C[a * d + b] : C[b * d + a];
    pi[j] = ps[j] / (double)n;
  }
  return ORC_OK;
}

int orc_em_train(int d, int64_t n, int k, const float *X, double *pi,
                 double *mu, double *sigma, int max_sweeps, double eps,
                 double abort_thr, double reg_coef, int svd,
                 double *logl_trace, double *e_trace, int *iter_counter,
                 double *final_logl, int nthreads) {
  return orc_em_train_order(d, n, k, X, pi, mu, sigma, max_sweeps, eps, abort_thr, reg_coef, svd, logl_trace,
                            e_trace, iter_counter, final_logl, nthreads, 0);
}

int orc_em_train_order(int d, int64_t n, int k, const float *X, double *pi,
                       double *mu, double *sigma, int max_sweeps, double eps,
                       double abort_thr, double reg_coef, int svd,
                       double *logl_trace, double *e_trace, int *iter_counter,
                       double *final_logl, int nthreads, int cached) {
  std::vector<double> U((size_t)k * d * d), logdet(k), post((size_t)n * k);
  double prev = -std::numeric_limits<double>::max(), logl = prev;
  int failed;
  auto cond_abort = [&]() {
    if (!svd) return false;
    double mx = 0.0;
    for (int j = 0; j < k; j++)
      mx = std::max(mx, orc_cond_number(d, sigma + (size_t)j * d * d));
    return mx > abort_thr;
  };
  orc_em_regularize(d, k, reg_coef, sigma);
  int st = orc_em_init_densities(d, k, sigma, U.data(), logdet.data(), &failed);
  if (st != ORC_OK) return st;
  if (cond_abort()) return ORC_ERR_COND_ABORT;
  int it;
  for (it = 1; it <= max_sweeps; it++) {
    orc_em_estep(d, n, k, X, pi, mu, U.data(), logdet.data(), post.data(), &logl, nthreads);
    if (cached)
      orc_em_mstep_cached(d, n, k, X, post.data(), pi, mu, sigma, nthreads);
    else
      orc_em_mstep(d, n, k, X, post.data(), pi, mu, sigma, nthreads);
    orc_em_regularize(d, k, reg_coef, sigma);
    st = orc_em_init_densities(d, k, sigma, U.data(), logdet.data(), &failed);
    if (st != ORC_OK) {
      if (iter_counter) *iter_counter = it;
      return st;
    }
    if (cond_abort()) {
      if (iter_counter) *iter_counter = it;
      return ORC_ERR_COND_ABORT;
    }
    double e = std::fabs((logl - prev) / logl);
    if (logl < prev) e = 0.0;
    if (logl_trace) logl_trace[it - 1] = logl;
    if (e_trace) e_trace[it - 1] = e;
    prev = logl;
    if (e < eps) {
      it++;
      break;
    }
  }
  if (iter_counter) *iter_counter = it;
  if (final_logl) *final_logl = logl;
  return ORC_OK;
}

/* ------------------------------------------------------------ k-means */

double orc_km_iterate(int d, int64_t n, int k, const float *X,
                      double *centroids, int64_t *counts, int32_t *labels,
                      int repair, int nthreads) {
  nthreads = resolve_threads(nthreads);
  const size_t kd = (size_t)k * d;
  std::vector<double> center((size_t)nthreads * kd, 0.0);
  std::vector<int64_t> cnt((size_t)nthreads * k, 0);
  std::vector<double> fitp(nthreads, 0.0);
#pragma omp parallel num_threads(nthreads)
  {
    int tid = omp_get_thread_num();
    int64_t off, c;
    find_items(n, nthreads, tid, off, c);
    double *myc = &center[(size_t)tid * kd];
    int64_t *myn = &cnt[(size_t)tid * k];
    std::vector<double> row(d);
    double fit = 0.0;
    for (int64_t i = off; i < off + c; i++) {
      const float *x = X + i * d;
      for (int q = 0; q < d; q++) row[q] = (double)x[q]; /* ConvertToOptFloat */
      double minssq = std::numeric_limits<double>::max();
      int bestj = -1;
      int j = 0;
      /* four independent accumulators, each summed in column order */
      for (; j + 4 <= k; j += 4) {
        const double *c0 = centroids + (size_t)j * d;
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        for (int q = 0; q < d; q++) {
          double t0 = c0[q] - row[q], t1 = c0[d + q] - row[q];
          double t2 = c0[2 * d + q] - row[q], t3 = c0[3 * d + q] - row[q];
          s0 += t0 * t0;
          s1 += t1 * t1;
          s2 += t2 * t2;
          s3 += t3 * t3;
        }
        if (s0 < minssq) { minssq = s0; bestj = j; }
        if (s1 < minssq) { minssq = s1; bestj = j + 1; }
        if (s2 < minssq) { minssq = s2; bestj = j + 2; }
        if (s3 < minssq) { minssq = s3; bestj = j + 3; }
      }
      for (; j < k; j++) {
        double s = sqdist_dd(d, centroids + (size_t)j * d, row.data());
        if (s < minssq) { minssq = s; bestj = j; }
      }
      fit += minssq;
      myn[bestj]++;
      double *cb = myc + (size_t)bestj * d;
      for (int q = 0; q < d; q++) cb[q] += row[q]; /* AddRow */
      if (labels) labels[i] = bestj;
    }
    fitp[tid] = fit;
  }
  /* Log2OpenMPReducer::ReduceToZero (Clust/OpenMPKMAReducer.cpp:162-179) */
  for (int s = 1; s < nthreads; s *= 2) {
    for (int t = 0; t < nthreads; t += 2 * s) {
      if (t + s < nthreads) {
        for (size_t q = 0; q < kd; q++) center[(size_t)t * kd + q] += center[(size_t)(t + s) * kd + q];
        for (int j = 0; j < k; j++) cnt[(size_t)t * k + j] += cnt[(size_t)(t + s) * k + j];
      }
    }
  }
  double fit = 0.0;
  for (int t = 0; t < nthreads; t++) fit += fitp[t];
  for (int j = 0; j < k; j++) {
    if (counts) counts[j] = cnt[j];
    if (cnt[j] > 0) {
      double f = 1.0 / (double)cnt[j];
      for (int q = 0; q < d; q++) centroids[(size_t)j * d + q] = center[(size_t)j * d + q] * f;
    } else if (repair) {
      /* CentroidRandomRepair::RepairVec */
      int64_t src = (int64_t)(orc_rng_uniform() * (double)n);
      for (int q = 0; q < d; q++) centroids[(size_t)j * d + q] = (double)X[src * d + q];
    }
  }
  return fit / (double)n;
}

double orc_km_run(int d, int64_t n, int k, const float *X, double *centroids,
                  double min_rel, int max_iter, int *iters, int nthreads) {
  double best = std::numeric_limits<double>::max();
  if (max_iter == 0) {
    if (iters) *iters = 0;
    return 0.0;
  }
  int i;
  for (i = 1;; i++) {
    double fit = orc_km_iterate(d, n, k, X, centroids, nullptr, nullptr, 1, nthreads);
    double rel = (best - fit) / best;
    if (fit < std::nextafter(fit, best))
      best = fit;
    else
      break;
    if (min_rel > 0.0 && min_rel > rel) break;
    if (max_iter > 0 && i == max_iter - 1) break;
  }
  if (iters) *iters = i;
  return best;
}

void orc_km_plusplus(int d, int64_t n, int k, const float *X,
                     const double *weights, double *vec) {
  std::vector<double> closest(n, std::numeric_limits<double>::infinity()), agg(n);
  int64_t first = (int64_t)(orc_rng_uniform() * (double)n);
  for (int q = 0; q < d; q++) vec[q] = X[first * d + q];
  for (int i = 1; i < k; i++) {
    const double *prev = vec + (size_t)(i - 1) * d;
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; j++) {
      double dist = sqdist_df(d, prev, X + j * d);
      if (closest[j] > dist) closest[j] = dist;
    }
    double sum = 0.0;
    for (int64_t j = 0; j < n; j++) {
      sum += closest[j] * (weights ? weights[j] : 1.0);
      agg[j] = sum;
    }
    for (int64_t j = 0; j < n; j++) agg[j] /= sum;
    double r = orc_rng_uniform();
    for (int64_t j = 0; j < n; j++) {
      if (r <= agg[j]) {
        for (int q = 0; q < d; q++) vec[(size_t)i * d + q] = X[j * d + q];
        break;
      }
    }
  }
}

void orc_km_oror(int d, int64_t n, int k, const float *X, double oversample,
                 double *vec, int nthreads) {
  nthreads = resolve_threads(nthreads);
  int rounds = (oversample <= 0.1) ? 10 : 5;
  std::vector<double> closest(n, std::numeric_limits<double>::infinity());
  std::vector<int> closest_c(n, -1);
  std::vector<float> centers; /* C x d */
  auto cost = [&]() {
    double s = 0.0;
    for (int64_t i = 0; i < n; i++) s += closest[i];
    return s;
  };
  /* InsertCentroid / InsertCentroids: per-row minimum over new centres */
  auto insert = [&](const std::vector<float> &nc) {
    int base = (int)(centers.size() / d);
    int m = (int)(nc.size() / d);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t i = 0; i < n; i++) {
      const float *row = X + i * d;
      for (int j = 0; j < m; j++) {
        double sq = sqdist_ff(d, &nc[(size_t)j * d], row);
        if (sq < closest[i]) {
          closest[i] = sq;
          closest_c[i] = base + j;
        }
      }
    }
    centers.insert(centers.end(), nc.begin(), nc.end());
  };
  int64_t first = (int64_t)(orc_rng_uniform() * (double)n);
  insert(std::vector<float>(X + first * d, X + first * d + d));
  double c = cost();
  for (int r = 0; r < rounds; r++) {
    std::vector<float> nc;
    /* ScanDataset on one thread: Rand() consumed in row order */
    for (int64_t i = 0; i < n; i++) {
      double prob = oversample * (double)k * closest[i] / c;
      if (orc_rng_uniform() < prob) nc.insert(nc.end(), X + i * d, X + i * d + d);
    }
    insert(nc);
    c = cost();
  }
  int64_t nc = (int64_t)(centers.size() / d);
  std::vector<double> w(nc, 0.0);
  for (int64_t i = 0; i < n; i++) w[closest_c[i]] += 1.0;
  orc_km_plusplus(d, nc, k, centers.data(), w.data(), vec);
}

void orc_km_forgy(int d, int64_t n, int k, const float *X, double *vec) {
  for (int i = 0; i < k; i++) {
    int64_t obj = (int64_t)(orc_rng_uniform() * (double)n);
    for (int q = 0; q < d; q++) vec[(size_t)i * d + q] = X[obj * d + q];
  }
}

}  // extern "C"
