/*
 * fastem_gpu.h -- C-ABI of the GB300 (sm_103a) EM and k-means hot path.
 *
 * The reference exposes this path as C++ virtual methods (no C ABI):
 *   EMAlgorithm        EM2/EMAlgorithm.h:26-79   (TrainNoCopy, SetParameters,
 *                      PrecomputeDensityMatrix, MStep, InitDensities, ...)
 *   SimpleMatrixEM     EM2/MatrixEM.h:83-100
 *   NormalDensity      EM2/NormalDensity.h:24-57
 *   KMeansAlgorithm    Clust/KMAlgorithm.h:29-68  (RunKMeans, ComputeMSEAndCorrect)
 *   NaiveKMA           Clust/KMAlgorithm.h:85-117
 * A CUDA backend registered beside "matrixem"/"simplematrixem"/"cachedem" in
 * CreateEMAlgorithm (EM2/EMAlgorithm.cpp:247-269) binds exactly these entry
 * points; the C++ classes in fastem_gb300/host/ are that binding.
 *
 * Conventions: plain pointers and sizes; N is int64_t; every array is
 * row-major; covariances are K consecutive d*d blocks; all parameters are
 * double on the host side (the reference's OPTFLOAT is double in every
 * build that compiles, Util/Optfloat.h:3-9).  Host pointers unless the name
 * says "device".  Every call returns a fem_status; the reference's
 * exceptions map as EMException -> FEM_ERR_CHOLESKY / FEM_ERR_COND_ABORT,
 * std::invalid_argument -> FEM_ERR_BAD_ARG.  A handle owns one CUDA stream
 * and must be used by one host thread at a time.  There is no CPU fallback:
 * without a usable CUDA device every create call returns FEM_ERR_NO_DEVICE.
 */
#ifndef FASTEM_GPU_H_
#define FASTEM_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FEM_API_VERSION 1

typedef enum fem_status {
  FEM_OK = 0,
  FEM_ERR_BAD_ARG = 1,     /* std::invalid_argument in the reference */
  FEM_ERR_CUDA = 2,        /* a CUDA runtime/driver call failed */
  FEM_ERR_CHOLESKY = 3,    /* "Cholesky decomposition failed" (EM2/NormalDensity.cpp:48-49) */
  FEM_ERR_COND_ABORT = 4,  /* "Condition number ... too high" (EM2/EMAlgorithm.cpp:147-151) */
  FEM_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
  FEM_ERR_NO_DEVICE = 6,   /* no CUDA device / not sm_103 */
  FEM_ERR_STATE = 7,       /* call out of order (e.g. iterate before upload) */
  FEM_ERR_UNSUPPORTED = 8  /* shape not supported by the requested precision */
} fem_status;

typedef enum fem_precision {
  FEM_PREC_FP64 = 0,  /* whole iteration in FP64, like the reference's double build */
  FEM_PREC_FP32 = 1,  /* whole iteration in FP32 on CUDA cores (plain baseline) */
  FEM_PREC_MIXED = 2  /* tcgen05 FP16 hi/lo split contractions, FP32 accumulate, FP64 Cholesky/logdet/logL */
} fem_precision;

/* returns FEM_API_VERSION */
int fem_api_version(void);
/* message of the last failing call on this thread (never NULL) */
const char *fem_last_error(void);

/* ================================ EM ================================= */

typedef struct fem_em fem_em;

typedef struct fem_em_config {
  int precision;      /* fem_precision */
  int device;         /* CUDA device ordinal */
  int max_sweeps;     /* EMAlgorithm::MaxSweeps   (default 1000000, EM2/EMAlgorithm.cpp:41) */
  double eps;         /* EMAlgorithm::Eps         (default 1e-5,    EM2/EMAlgorithm.cpp:42) */
  double abort_thr;   /* EMAlgorithm::AbortThr    (default 1e5,     EM2/EMAlgorithm.cpp:43) */
  double reg_coef;    /* EMAlgorithm::RegCoef     (default 0,       EM2/EMAlgorithm.cpp:44) */
  int svd;            /* condition-number check per sweep (EM2/EMArgs.cpp:40, default on) */
} fem_em_config;

/* fills the reference defaults (precision FEM_PREC_MIXED, device 0) */
void fem_em_config_default(fem_em_config *cfg);

/* EMAlgorithm / SimpleMatrixEM constructor (EM2/EMAlgorithm.cpp:32-64,
 * EM2/MatrixEM.cpp:259-273): sizes every device buffer for n rows, d
 * columns and k components.  Replaces CreateEMAlgorithm("simplematrixem",
 * ...) (EM2/EMAlgorithm.cpp:247-269). */
int fem_em_create(int d, int64_t n, int k, const fem_em_config *cfg, fem_em **out);
void fem_em_destroy(fem_em *h);

/* EMAlgorithm::SetParameters (EM2/EMAlgorithm.cpp:25-30) */
int fem_em_set_parameters(fem_em *h, int max_sweeps, double eps, double abort_thr,
                          double reg_coef);

/* EMAlgorithm::CopyDataset / MatrixEM::CopyDataset (EM2/EMAlgorithm.cpp:225-235,
 * EM2/MatrixEM.cpp:102-121): float rows (ld floats apart) -> device. */
int fem_em_upload(fem_em *h, const float *X, int64_t ld);
/* same, from device memory (rows already resident in HBM) */
int fem_em_upload_device(fem_em *h, const float *dX, int64_t ld);

/* EMAlgorithm::DecodeMixture (EM2/EMAlgorithm.cpp:125-131): pi[k], mu[k*d],
 * sigma[k*d*d] (the lower triangle is used, EM2/NormalDensity.cpp:45). */
int fem_em_set_params(fem_em *h, const double *pi, const double *mu, const double *sigma);
/* GaussianMixture::Init target of TrainNoCopy (EM2/EMAlgorithm.cpp:186-189) */
int fem_em_get_params(fem_em *h, double *pi, double *mu, double *sigma);

/* EMAlgorithm::TrainNoCopy (EM2/EMAlgorithm.cpp:139-191): regularise,
 * factor, optional condition check, then sweeps until |dL/L| < Eps or
 * MaxSweeps.  logl_trace / e_trace (capacity entries each, may be NULL)
 * receive the per-sweep LogL and e; *iter_counter is IterCounter after the
 * loop; *logl the returned LogL (computed before the last M-step). */
int fem_em_train(fem_em *h, int svd, double *logl_trace, double *e_trace, int capacity,
                 int *iter_counter, double *logl);

/* Single pieces of one sweep, for hosts that drive the loop themselves:
 * EMAlgorithm::InitDensities after RegularizeCovariances
 * (EM2/EMAlgorithm.cpp:75-87,237-244); status FEM_ERR_CHOLESKY with the
 * failing component in *failed. */
int fem_em_init_densities(fem_em *h, int *failed);
/* SimpleMatrixEM::PrecomputeDensityMatrix + ComputeLogLike
 * (EM2/MatrixEM.cpp:275-307): posteriors on device, returns sum_i LSE_i */
int fem_em_precompute(fem_em *h, double *logl);
/* SimpleMatrixEM::MStep (EM2/MatrixEM.cpp:309-378) */
int fem_em_mstep(fem_em *h);
/* EMAlgorithm::FindLargestConditionNumber (EM2/EMAlgorithm.cpp:193-202) */
int fem_em_max_condition(fem_em *h, double *cond);

/* Self-test of the bounded device waits (no counterpart in the reference,
 * whose CPU loops have no device waits to bound; the reference's failure
 * path it stands beside is the EMException of EM2/EMAlgorithm.cpp:147-163).
 * Runs one small kernel with the roles of the mixed-precision kernels (a
 * producer that never delivers, a consumer, a drain, two waiters off the
 * critical path) whose waits give up after `budget_cycles` (1e3 .. 4e9):
 * returns FEM_ERR_TIMEOUT with the message the real kernels' expiry produces,
 * and *roles = bit mask of the waits that gave up (1 consumer, 2 drain, 4 and
 * 8 the waiters that left on the status word).  The handle stays usable: the
 * next call starts with the status word cleared.  Mixed-precision handles
 * only (FEM_ERR_UNSUPPORTED otherwise). */
int fem_em_selftest_wait_expiry(fem_em *h, int64_t budget_cycles, int *roles);

/* EMAlgorithm::Posteriors (EM2/EMAlgorithm.h:41) after the last E-step, as
 * an n x k row-major double matrix. */
int fem_em_get_posteriors(fem_em *h, double *post);
/* EMAlgorithm::RetrieveClasses (EM2/EMAlgorithm.cpp:107-122) */
int fem_em_retrieve_classes(fem_em *h, int32_t *classes);
/* EMAlgorithm::ComputePosterriorCorrelation (EM2/EMAlgorithm.cpp:213-219):
 * corr = R^T R (k x k, row-major) over the posteriors of the last E-step,
 * computed on the device */
int fem_em_posterior_correlation(fem_em *h, double *corr);
/* NormalDensity::GetInvertedCholCov / GetLogDeterminant
 * (EM2/NormalDensity.h:42,45): U_j = (L_j^-1)^T upper, k*d*d, and logdet[k] */
int fem_em_get_factors(fem_em *h, double *U, double *logdet);

/* Device time (ms, CUDA events on the handle's stream) of the E-step and
 * M-step kernels over the last `fem_em_timing_reset` window, and launch
 * counts. */
int fem_em_timing_reset(fem_em *h, int enable);
int fem_em_timing_get(fem_em *h, double *estep_ms, double *mstep_ms, double *finalize_ms,
                      int64_t *launches);
/* device time (ms) from the first to the last kernel of every
 * fem_em_train sweep loop since the last reset, and the sweeps it ran */
int fem_em_timing_total(fem_em *h, double *train_ms, int64_t *sweeps);
/* device time (ms) of the mixed-precision covariance kernel alone (the
 * rank-update part of EM2/MatrixEM.cpp:90-99) since the last reset */
int fem_em_timing_covariance(fem_em *h, double *cov_ms);

/* =========================== batched EM ============================== */

/* Many independent fits trained together on one GPU.  No single reference
 * counterpart: the reference trains one mixture per em2 run (EM2/main.cpp),
 * and each fit here follows that run's loop, EMAlgorithm::TrainNoCopy
 * (EM2/EMAlgorithm.cpp:139-191) with the SimpleMatrixEM sweep
 * (EM2/MatrixEM.cpp:275-378), on its own data, with its own convergence test
 * and failure status.  Every kernel of a sweep covers all fits still
 * sweeping.  FEM_PREC_FP32: FP32 on CUDA cores with FP64 partial sums,
 * factorisation and LogL (cfg NULL: the reference defaults with FP32).
 * FEM_PREC_MIXED: the same, except that the E-step of the fits with
 * 16 < d <= 32 runs on the tensor cores (FP16 x 3 split products, FP32
 * accumulation).  Per fit d <= 32, k <= 64, n < 2^31 (larger shapes:
 * FEM_ERR_UNSUPPORTED). */
typedef struct fem_em_batch fem_em_batch;

int fem_em_batch_create(int nfits, const int *d, const int64_t *n, const int *k,
                        const fem_em_config *cfg, fem_em_batch **out);
/* Work-item sizes per dimension class (d <= 4, 8, 16, 32): points per means
 * item and per covariance item (multiples of 128 in [256, 16384]).  The
 * engine has no reference counterpart; the sizes change the schedule and the
 * order of the FP32 item sums, not the sweep.  fastem_gb300/autotune.py
 * measures them on a GPU and writes the table that CudaBatchEM loads. */
typedef struct {
  int means_chunk[4];
  int cov_chunk[4];
} fem_em_batch_tuning;
void fem_em_batch_tuning_default(fem_em_batch_tuning *t);
/* fem_em_batch_create with the item sizes of `tuning` (NULL: the defaults) */
int fem_em_batch_create_tuned(int nfits, const int *d, const int64_t *n, const int *k,
                              const fem_em_config *cfg, const fem_em_batch_tuning *tuning,
                              fem_em_batch **out);
/* the item sizes a batch was created with */
int fem_em_batch_get_tuning(fem_em_batch *b, fem_em_batch_tuning *t);
void fem_em_batch_destroy(fem_em_batch *b);
/* EMAlgorithm::SetParameters (EM2/EMAlgorithm.cpp:25-30), for every fit */
int fem_em_batch_set_parameters(fem_em_batch *b, int max_sweeps, double eps, double abort_thr,
                                double reg_coef);
/* fit `fit`'s n x d float rows, ld floats apart (EM2/EMAlgorithm.cpp:225-235) */
int fem_em_batch_upload(fem_em_batch *b, int fit, const float *X, int64_t ld);
/* every fit's rows, packed one fit after another (fit 0's n0 x d0, then fit 1's ...) */
int fem_em_batch_upload_packed(fem_em_batch *b, const float *X);
/* EMAlgorithm::DecodeMixture (EM2/EMAlgorithm.cpp:125-131) for one fit */
int fem_em_batch_set_params(fem_em_batch *b, int fit, const double *pi, const double *mu,
                            const double *sigma);
int fem_em_batch_get_params(fem_em_batch *b, int fit, double *pi, double *mu, double *sigma);
/* trains every fit.  Per fit (arrays of nfits, each may be NULL): status is
 * FEM_OK, FEM_ERR_CHOLESKY or FEM_ERR_COND_ABORT (what fem_em_train would
 * return for that fit alone), iter_counter its IterCounter, logl its last
 * LogL.  Returns FEM_OK when the batch ran, whatever the fits' statuses. */
int fem_em_batch_train(fem_em_batch *b, int svd, int *status, int *iter_counter, double *logl);
/* per-sweep LogL and e of one fit's last train (the first min(capacity,
 * max_sweeps, 4096) sweeps) */
int fem_em_batch_trace(fem_em_batch *b, int fit, double *logl_trace, double *e_trace, int capacity);
/* the component whose Cholesky factorisation stopped the fit (-1: none) */
int fem_em_batch_fail_component(fem_em_batch *b, int fit, int *component);
/* per-phase device time (ms, CUDA events): [0] E-step, [1] means and their
 * reduction, [2] covariance sums, [3] reduction + factorisation + sweep end,
 * [4] the whole sweep loop; kernel launches and sweeps since enabling */
int fem_em_batch_timing_enable(fem_em_batch *b, int on);
int fem_em_batch_timing(fem_em_batch *b, double *phase_ms, int64_t *launches, int64_t *sweeps);
/* the E-step, means and covariance launches of each dimension class (d <= 4, 8, 16,
 * 32) since enabling: class_ms[3 * 4], [phase * 4 + class] (ms, CUDA events) */
int fem_em_batch_timing_classes(fem_em_batch *b, double *class_ms);

/* ============================== k-means ============================== */

typedef struct fem_km fem_km;

enum { FEM_KM_REPAIR_NONE = 0, FEM_KM_REPAIR_RANDOM = 1, FEM_KM_REPAIR_NEXT = 2 };

typedef struct fem_km_config {
  int precision;   /* FEM_PREC_FP32 (CUDA-core distances) or FEM_PREC_MIXED (tcgen05, FP16 hi/lo splits) */
  int device;
  uint64_t seed;   /* seed of the repair RNG (Util/Rand.cpp SRand) */
  int repair;      /* an empty cluster's centroid becomes: FEM_KM_REPAIR_RANDOM the row at Rand() * N
                      (CentroidRandomRepair, Clust/CentroidRepair.cpp:21-28); FEM_KM_REPAIR_NEXT rows
                      0, 1, 2, ... in turn, wrapping at N, one counter per handle
                      (CentroidDeterministicRepair, :30-43); FEM_KM_REPAIR_NONE unchanged */
} fem_km_config;

void fem_km_config_default(fem_km_config *cfg);

/* NaiveKMA constructor (Clust/KMAlgorithm.cpp:102-115) */
int fem_km_create(int d, int64_t n, int k, const fem_km_config *cfg, fem_km **out);
void fem_km_destroy(fem_km *h);
/* rows of the MultithreadedDataset the reference iterates over */
int fem_km_upload(fem_km *h, const float *X, int64_t ld);
int fem_km_upload_device(fem_km *h, const float *dX, int64_t ld);
/* NaiveKMA::InitDataStructures (Clust/KMAlgorithm.cpp:140-146) */
int fem_km_init_data_structures(fem_km *h);
/* NaiveKMA::ComputeMSEAndCorrect (Clust/KMAlgorithm.cpp:205-255):
 * centroids (k*d double, CentroidVector layout Clust/CentroidVector.h:11-17)
 * updated in place; *fit = sum of squared distances / N; counts[k] may be
 * NULL.  Assignments are bit-exact to an FP64 difference-form argmin with
 * the lowest index winning ties. */
int fem_km_compute_mse_and_correct(fem_km *h, double *centroids, double *fit, int64_t *counts);
/* NaiveKMA::CorrectWithoutMSE (Clust/KMAlgorithm.cpp:148-202): the same
 * iteration without the fit; *changed = 1 when some point's label differs
 * from the one stored by the previous iteration (all zero after
 * fem_km_init_data_structures, like Assignment[]) */
int fem_km_correct_without_mse(fem_km *h, double *centroids, int *changed);
/* KMeansAlgorithm::RunKMeans (Clust/KMAlgorithm.cpp:44-87) */
int fem_km_run(fem_km *h, double *centroids, double min_rel, int max_iter, double *best_fit,
               int *iters);
/* assignment of every row after the last iteration */
int fem_km_get_assignment(fem_km *h, int32_t *labels);
/* reseed the repair RNG (SRand, Util/Rand.cpp:33-35) */
int fem_km_seed(fem_km *h, uint64_t seed);
/* The reference repairs empty clusters from its one global Rand() stream
 * (Util/Rand.cpp:7-14, Clust/CentroidRepair.cpp:21-28), which the seeding
 * drew from first.  These copy the repair RNG's std::mt19937_64 state in and
 * out as the text the C++ standard library's stream operators write, so a
 * host that seeds with its own generator continues the same stream.
 * fem_km_get_rng_state needs len > the text's length (about 7 KB;
 * FEM_KM_RNG_STATE_LEN is enough). */
#define FEM_KM_RNG_STATE_LEN 8192
int fem_km_set_rng_state(fem_km *h, const char *state);
int fem_km_get_rng_state(fem_km *h, char *buf, size_t len);

/* k-means classification that allocates nothing.  No counterpart in the
 * reference: a handle-free variant of the assignment kernel with the
 * semantics of CentroidVector::ClassifyDataset + ComputeMSE
 * (Clust/CentroidVector.cpp:8-34,56-94), for callers that must not allocate
 * device memory once running.  dX (n x d float, row-major), dCent (k x d
 * double), dLabels (n int32) and dFit (one double: sum of squared distances
 * / n) are caller-owned device buffers on `device`; `stream` is a
 * cudaStream_t (NULL: the default stream); the call is asynchronous.
 * Scratch is one fixed 140 KiB __device__ array: k <= 1024, k*d <= 32768,
 * d in {2,4,8,16,32,64}; larger k fail with FEM_ERR_BAD_ARG.  The first call
 * on a device does the set-up (resolves the array's address) and should
 * precede any stream capture.  Every call on a device shares the array: it
 * keeps the last call's contents, nothing in it has to start at zero, and
 * calls that overlap in time race. */
int fem_km_classify_noalloc(int d, int64_t n, int k, const float *dX, const double *dCent,
                            int32_t *dLabels, double *dFit, int device, void *stream);
/* diagnostics: rows re-decided in FP64 and kernel time of the last iteration */
int fem_km_stats(fem_km *h, int64_t *rechecked_rows, double *assign_ms, double *update_ms);

#ifdef __cplusplus
}
#endif

#endif /* FASTEM_GPU_H_ */
