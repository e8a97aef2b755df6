/*
 * fem_oracle.h -- FP64 CPU restatement of FastEM's EM and k-means hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code: it is the checker that the CUDA path is compared against
 * (tests/, __graft_entry__.smoke()) and the timed CPU baseline (bench.py's
 * cpu_baseline leg and its --impl reference arm).
 *
 * PARITY UNPINNED.  The reference (wkwedlo/fastem) cannot be compiled in this
 * environment (it needs Eigen 3.4, Intel MKL, libnuma and MPI, none of which
 * are present) and it ships no tests, golden vectors or fixtures.  This
 * restatement is therefore pinned only against an independent numpy/scipy
 * FP64 computation (tests/test_oracle.py) and against the golden fixtures it
 * produced itself (tests/golden/).
 *
 * Every function below names the reference routine it restates.  All arrays
 * are row-major; covariance and factor matrices are K consecutive d*d blocks.
 */
#ifndef FEM_ORACLE_H_
#define FEM_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (same values as include/fastem_gpu.h) */
#define ORC_OK 0
#define ORC_ERR_BAD_ARG 1
#define ORC_ERR_CHOLESKY 3
#define ORC_ERR_COND_ABORT 4

/* ---- global RNG: one std::mt19937_64 + uniform_real_distribution<double>,
 *      like Util/Rand.cpp:7-36 (SRand / Rand). ---- */
void orc_rng_seed(uint64_t seed);
double orc_rng_uniform(void);

/* ---- EM ---------------------------------------------------------------- */

/* NormalDensity::Init (EM2/NormalDensity.cpp:43-65) for K components:
 * C = sym(lower(sigma_j)), L = chol(C), logdet_j = 2 sum log L_ii,
 * U_j = (L^-1)^T (upper triangular, row-major).  Returns ORC_ERR_CHOLESKY
 * and the first failing component in *failed when a pivot is <= 0. */
int orc_em_init_densities(int d, int k, const double *sigma, double *U,
                          double *logdet, int *failed);

/* EMAlgorithm::RegularizeCovariances (EM2/EMAlgorithm.cpp:237-244). */
void orc_em_regularize(int d, int k, double reg_coef, double *sigma);

/* NormalDensity::ComputeConditionNumber (EM2/NormalDensity.cpp:67-71):
 * |lambda_max / lambda_min| of sym(lower(sigma)), cyclic Jacobi. */
double orc_cond_number(int d, const double *sigma);

/* SimpleMatrixEM::PrecomputeDensityMatrix (EM2/MatrixEM.cpp:275-307) with
 * BlockDensities (:69-81), CalcLogCoeffs (:83-87) and
 * PostProcessDensityMatrix (:39-51).  post is N x K; *logl = sum_i LSE_i. */
int orc_em_estep(int d, int64_t n, int k, const float *X, const double *pi,
                 const double *mu, const double *U, const double *logdet,
                 double *post, double *logl, int nthreads);

/* SimpleMatrixEM::doMStep (EM2/MatrixEM.cpp:309-378): PosteriorSum, means
 * by R^T X, covariances by the sqrt(r)/sqrt(N_j)-weighted rank-k update
 * around the new means, upper mirrored to lower, pi = PosteriorSum / N. */
int orc_em_mstep(int d, int64_t n, int k, const float *X, const double *post,
                 double *pi, double *mu, double *sigma, int nthreads);

/* CachedEM::MStep (EM2/CachedEM.cpp:88-170): the same means and posterior
 * sums, covariances as rank-1 updates weighted by the unscaled posteriors
 * around the new means, divided by the posterior sum after the reduction
 * (SimpleMatrixEM scales every point by sqrt(r / N_j) first). */
int orc_em_mstep_cached(int d, int64_t n, int k, const float *X, const double *post,
                        double *pi, double *mu, double *sigma, int nthreads);

/* EMAlgorithm::TrainNoCopy (EM2/EMAlgorithm.cpp:139-191) driving
 * SimpleMatrixEM.  pi/mu/sigma hold the initial mixture on entry and the
 * final one on return.  logl_trace/e_trace receive one value per sweep
 * (capacity max_sweeps, may be NULL).  *iter_counter is IterCounter after
 * the loop (the reference prints IterCounter-1 sweeps).  Returns the
 * LogL of the last sweep in *final_logl. */
int orc_em_train(int d, int64_t n, int k, const float *X, double *pi,
                 double *mu, double *sigma, int max_sweeps, double eps,
                 double abort_thr, double reg_coef, int svd,
                 double *logl_trace, double *e_trace, int *iter_counter,
                 double *final_logl, int nthreads);

/* orc_em_train with the M-step order chosen: cached = 0 SimpleMatrixEM
 * (orc_em_mstep), 1 CachedEM (orc_em_mstep_cached). */
int orc_em_train_order(int d, int64_t n, int k, const float *X, double *pi,
                       double *mu, double *sigma, int max_sweeps, double eps,
                       double abort_thr, double reg_coef, int svd,
                       double *logl_trace, double *e_trace, int *iter_counter,
                       double *final_logl, int nthreads, int cached);

/* ---- k-means ----------------------------------------------------------- */

/* NaiveKMA::ComputeMSEAndCorrect (Clust/KMAlgorithm.cpp:205-255) with
 * CentroidVector::SquaredDistance (Clust/CentroidVector.h:90-102) and
 * AddRow (:51-60).  centroids (K x d) are updated in place; empty clusters
 * are repaired with CentroidRandomRepair (Clust/CentroidRepair.cpp:21-28)
 * drawing from the global RNG when repair != 0.  counts/labels may be NULL.
 * Returns fit / N. */
double orc_km_iterate(int d, int64_t n, int k, const float *X,
                      double *centroids, int64_t *counts, int32_t *labels,
                      int repair, int nthreads);

/* KMeansAlgorithm::RunKMeans (Clust/KMAlgorithm.cpp:44-87).  Returns
 * BestFit; *iters receives i at loop exit. */
double orc_km_run(int d, int64_t n, int k, const float *X, double *centroids,
                  double min_rel, int max_iter, int *iters, int nthreads);

/* PlusPlusInitializer::Init (Clust/PlusPlusInitializer/PlusPlusInitializer.cpp:33-83)
 * over rows X (weights NULL = all 1). Draws from the global RNG. */
void orc_km_plusplus(int d, int64_t n, int k, const float *X,
                     const double *weights, double *centroids);

/* KMeansOrOrInitializer::Init (Clust/KMeansOrOrInitializer.cpp:143-174),
 * ScanDataset run on one thread so the global RNG is consumed in row order. */
void orc_km_oror(int d, int64_t n, int k, const float *X, double oversample,
                 double *centroids, int nthreads);

/* ForgyInitializer::Init (Clust/KMeansInitializer.cpp:33-49). */
void orc_km_forgy(int d, int64_t n, int k, const float *X, double *centroids);

/* One sweep (factorise, E-step with logL, M-step) organised like
 * SimpleMatrixEM with level-3 BLAS: for CPU timing (fem_oracle_blas.cpp).  The
 * CBLAS dtrmm / dgemm / dsyrk entry points are supplied by the caller.
 * pi, mu, sigma are updated in place; *logl is the pre-M-step logL. */
int orc_em_sweep_blas(int d, int64_t n, int k, const float *X, double *pi, double *mu, double *sigma,
                      double *logl, int nthreads, void *dtrmm, void *dgemm, void *dsyrk);
int orc_em_sweeps_blas(int d, int64_t n, int k, const float *X, double *pi, double *mu, double *sigma,
                       int sweeps, int svd, double abort_thr, double *logl, double *seconds, int nthreads,
                       void *dtrmm, void *dgemm, void *dsyrk);

#ifdef __cplusplus
}
#endif

#endif
