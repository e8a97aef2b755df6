// fastem.hpp -- C++ host classes mirroring the reference's interfaces on top
// of the C-ABI (include/fastem_gpu.h):
//
//   Dataset          MultithreadedDataset (.bin files, Util/MultithreadedDataset.cpp:119-134)
//   GaussianMixture  EM2/GaussianMixture.h:17-58 (.cmp files, EM2/GaussianMixture.cpp:155-171,228-244)
//   CudaEM           EMAlgorithm (EM2/EMAlgorithm.h:26-79) running on one GB300
//   CudaKMeans       KMeansAlgorithm (Clust/KMAlgorithm.h:30-75) running on one GB300
//   initialisers     EM2/EMInitializer.cpp:37-177 (jain, kmeans, kmeansoror, file)
//
// Errors are thrown as the reference throws them: EMException for numerical
// failures (EM2/EMException.h), FileException for I/O (Util/FileException.h),
// std::invalid_argument for bad arguments, std::runtime_error otherwise.
#pragma once

#include <cstdint>
#include <cstdio>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "fastem_gpu.h"

namespace fastem {

struct EMException : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct FileException : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// status of a C-ABI call -> the reference's exception types
void check(int status);

// ------------------------------------------------------------------ data
class Dataset {
 public:
  Dataset() = default;
  Dataset(int64_t rows, int cols) : nRows(rows), nCols(cols), data((size_t)rows * cols) {}
  // .bin: int32 rows (or -1 then int64 rows), int32 cols, rows of float32
  static Dataset Load(const char *fname);
  void Save(const char *fname) const;
  int64_t GetRowCount() const { return nRows; }
  int GetColCount() const { return nCols; }
  const float *GetRow(int64_t i) const { return data.data() + (size_t)i * nCols; }
  float *GetRow(int64_t i) { return data.data() + (size_t)i * nCols; }
  const float *Data() const { return data.data(); }
  // trace of the data covariance matrix (JainEMInitializer, EM2/EMInitializer.cpp:39)
  double GetCovMatrixTrace() const;

 private:
  int64_t nRows = 0;
  int nCols = 0;
  std::vector<float> data;
};

// --------------------------------------------------------------- mixture
class GaussianMixture {
 public:
  GaussianMixture() = default;
  GaussianMixture(int components, int cols);
  // .cmp: int32 K, int32 d, per component d*d covariance (row-major), d
  // mean, weight (all FP64), then one FP64 log-likelihood
  static GaussianMixture Read(const char *fname);
  static GaussianMixture Read(FILE *f);
  void Write(const char *fname, double loglike = 0.0) const;
  void Write(FILE *f, double loglike = 0.0) const;

  // GaussianMixture::Init(Weights, Covs, Means)
  void Init(const std::vector<double> &weights, const std::vector<double> &covs, const std::vector<double> &means);
  int GetComponentCount() const { return K; }
  int GetDimension() const { return d; }
  double GetWeight(int j) const { return weights[j]; }
  const double *GetMean(int j) const { return means.data() + (size_t)j * d; }
  const double *GetCovariance(int j) const { return covs.data() + (size_t)j * d * d; }
  std::vector<double> &Weights() { return weights; }
  std::vector<double> &Means() { return means; }
  std::vector<double> &Covs() { return covs; }
  const std::vector<double> &Weights() const { return weights; }
  const std::vector<double> &Means() const { return means; }
  const std::vector<double> &Covs() const { return covs; }

  // the mixture density sum_j pi_j N(x; mu_j, Sigma_j) and the argmax_j of
  // its terms, lowest index on ties (GaussianMixture::Evaluate / Classify,
  // EM2/GaussianMixture.cpp:54-98), FP64 on the host, one Cholesky per
  // component on first use.  Both work in the log domain: where every
  // density underflows to 0 (a row far from all components) the reference's
  // Classify returns 0, this one the component of largest log(pi_j N(x))
  double Evaluate(const float *x) const;
  int Classify(const float *x) const;

  // largest lambda_max / lambda_min over the components' covariances
  // (GaussianMixture::FindLargestConditionNumber, EM2/GaussianMixture.cpp;
  // NormalDensity::ComputeConditionNumber, EM2/NormalDensity.cpp:67-71):
  // eigenvalues by cyclic Jacobi in FP64 on the host
  double FindLargestConditionNumber() const;
  // the components' weights, means and covariances, then the condition
  // number, as GaussianMixture::Dump (EM2/GaussianMixture.cpp:139-153) prints them
  void Dump(FILE *f = stdout) const;

 private:
  void Factor() const;
  double LogDensities(const float *x, std::vector<double> &l) const;
  int K = 0, d = 0;
  std::vector<double> weights, means, covs;
  mutable std::vector<double> chol, logc;   // lower factors and log coefficients
};

// ---------------------------------------------------------------------- EM
class CudaEM {
 public:
  // precision: FEM_PREC_MIXED (default), FEM_PREC_FP32 or FEM_PREC_FP64
  CudaEM(int ncols, int64_t nrows, int ncl, int precision = FEM_PREC_MIXED, int device = 0);
  ~CudaEM();
  CudaEM(const CudaEM &) = delete;
  CudaEM &operator=(const CudaEM &) = delete;

  void SetParameters(int maxSweeps, double eps, double abortThr, double regCoef = 0.0);
  void CopyDataset(const Dataset &data);
  // EMAlgorithm::Train / TrainNoCopy: returns the log-likelihood before the
  // last M-step; G is replaced by the fitted mixture
  double Train(const Dataset &data, GaussianMixture &G, int verbosity, bool svd);
  double TrainNoCopy(GaussianMixture &G, int verbosity, bool svd);
  int GetIterCounter() const { return iterCounter; }
  void ClearIterCounter() { iterCounter = 0; }
  int GetK() const { return K; }
  const std::vector<double> &LogLikeTrace() const { return logl; }
  void RetrieveClasses(std::vector<int32_t> &classes) const;
  // EMAlgorithm::ComputePosterriorCorrelation (EM2/EMAlgorithm.cpp:213-219):
  // R^T R (K x K, row-major) over the posteriors of the last E-step
  void ComputePosterriorCorrelation(std::vector<double> &corr) const;
  const char *GetName() const;
  fem_em *Handle() const { return h; }

 private:
  fem_em *h = nullptr;
  int nCols, K, maxSweeps = 1000000;
  int64_t nRows;
  int iterCounter = 0;
  std::vector<double> logl, e;
};

// ---------------------------------------------------------------- k-means
class CudaKMeans {
 public:
  CudaKMeans(const Dataset &data, int nclusters, int precision = FEM_PREC_MIXED, int device = 0,
             uint64_t seed = 0, bool repair = true);
  ~CudaKMeans();
  CudaKMeans(const CudaKMeans &) = delete;
  CudaKMeans &operator=(const CudaKMeans &) = delete;

  // KMeansAlgorithm::RunKMeans: returns the best fit; vec is K*d centroids
  double RunKMeans(std::vector<double> &vec, int verbosity, double minRel = -1.0, int maxIter = 0);
  double ComputeMSEAndCorrect(std::vector<double> &vec);
  void InitDataStructures();
  int GetIterCount() const { return iterCount; }
  void Assignment(std::vector<int32_t> &labels) const;
  // repairs continue the caller's Rand() stream (the reference's one global
  // generator): copy its state in before and back out after the iterations
  void SetRngState(const std::string &state);
  std::string GetRngState() const;

 private:
  fem_km *h = nullptr;
  int64_t nRows;
  int nCols, K;
  int iterCount = 0;
};

// ------------------------------------------------------------ initialisers
// the reference's Rand(): one mt19937_64 stream, uniform [0, 1)
class Rand {
 public:
  explicit Rand(uint64_t seed) : rng(seed) {}
  double operator()() { return uni(rng); }
  // the generator's state as the standard library's stream operators write it
  std::string State() const;
  void SetState(const std::string &state);

 private:
  std::mt19937_64 rng;
  std::uniform_real_distribution<> uni;
};

// Forgy centroids (ForgyInitializer::Init, Clust/KMeansInitializer.cpp:33-49):
// K rows at Rand() * N, repeats allowed
std::vector<double> Forgy(const Dataset &data, int K, Rand &rnd);
// k-means++ centroids (Clust/PlusPlusInitializer/PlusPlusInitializer.cpp:33-83),
// FP64 on the host over `sample` rows spread evenly over the dataset (all rows,
// as the reference, if sample <= 0 or >= N)
std::vector<double> KMeansPlusPlus(const Dataset &data, int K, Rand &rnd, int64_t sample = 0);
// weighted k-means++ over M candidate rows P (PlusPlusInitializer with
// SetWeights: first row uniform, then D^2 w sampling), w may be null
std::vector<double> WeightedPlusPlus(const float *P, int64_t M, int d, const double *w, int K, Rand &rnd);
// k-means|| centroids (Clust/KMeansOrOrInitializer.cpp:143-174): a random first
// row, 5 rounds (10 if oversample <= 0.1) sampling each row with probability
// oversample K D^2 / cost, the candidates weighted by the rows closest to them,
// then weighted k-means++ down to K.  The sampling pass draws in row order (the
// reference's multi-threaded pass shares one generator between threads)
std::vector<double> KMeansOrOr(const Dataset &data, int K, Rand &rnd, double oversample = 1.4);
// initial mixture by name: "jain", "kmeans", "kmeansoror" or a .cmp file
// (CreateEMInitializer, EM2/EMInitializer.cpp:168-177)
GaussianMixture InitMixture(const char *name, const Dataset &data, int K, Rand &rnd, int precision = FEM_PREC_MIXED,
                            int device = 0);

}  // namespace fastem
