// fastem.cpp -- host classes of fastem.hpp over the C-ABI.
#include "fastem.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <sstream>
#include <thread>
#include <unordered_set>

namespace fastem {

void check(int st) {
  if (st == FEM_OK) return;
  const std::string msg = fem_last_error();
  if (st == FEM_ERR_CHOLESKY || st == FEM_ERR_COND_ABORT) throw EMException(msg);
  if (st == FEM_ERR_BAD_ARG) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

namespace {

// rows [0, n) split over the host threads; f(begin, end, thread)
template <class F>
void parallel_rows(int64_t n, F f) {
  const int nt = (int)std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++) {
    const int64_t b = n * t / nt, e = n * (t + 1) / nt;
    th.emplace_back([=, &f] { f(b, e, t); });
  }
  for (auto &x : th) x.join();
}

int host_threads() { return (int)std::max(1u, std::min(64u, std::thread::hardware_concurrency())); }

}  // namespace

// ------------------------------------------------------------------ data
Dataset Dataset::Load(const char *fname) {
  FILE *f = std::fopen(fname, "rb");
  if (!f) throw FileException(std::string("cannot open ") + fname);
  int32_t r32 = 0, c32 = 0;
  int64_t rows = 0;
  if (std::fread(&r32, 4, 1, f) != 1 || std::fread(&c32, 4, 1, f) != 1) {
    std::fclose(f);
    throw FileException("read failed");
  }
  if (r32 == -1) {
    if (std::fread(&rows, 8, 1, f) != 1) {
      std::fclose(f);
      throw FileException("read failed");
    }
  } else {
    rows = r32;
  }
  if (rows < 0 || c32 <= 0) {
    std::fclose(f);
    throw FileException("invalid .bin header");
  }
  Dataset D(rows, c32);
  const size_t want = (size_t)rows * c32;
  if (std::fread(D.data.data(), sizeof(float), want, f) != want) {
    std::fclose(f);
    throw FileException("Invalid number of bytes read");
  }
  std::fclose(f);
  return D;
}

void Dataset::Save(const char *fname) const {
  FILE *f = std::fopen(fname, "wb");
  if (!f) throw FileException(std::string("cannot create ") + fname);
  bool ok;
  if (nRows <= INT32_MAX) {
    const int32_t r = (int32_t)nRows, c = nCols;
    ok = std::fwrite(&r, 4, 1, f) == 1 && std::fwrite(&c, 4, 1, f) == 1;
  } else {
    const int32_t m = -1, c = nCols;
    ok = std::fwrite(&m, 4, 1, f) == 1 && std::fwrite(&c, 4, 1, f) == 1 && std::fwrite(&nRows, 8, 1, f) == 1;
  }
  ok = ok && std::fwrite(data.data(), sizeof(float), data.size(), f) == data.size();
  std::fclose(f);
  if (!ok) throw FileException("write failed");
}

double Dataset::GetCovMatrixTrace() const {
  if (nRows < 2) return 0.0;
  const int nt = host_threads();
  std::vector<double> s1((size_t)nt * nCols, 0.0), s2((size_t)nt * nCols, 0.0);
  parallel_rows(nRows, [&](int64_t b, int64_t e, int t) {
    double *a = s1.data() + (size_t)t * nCols, *q = s2.data() + (size_t)t * nCols;
    for (int64_t i = b; i < e; i++)
      for (int c = 0; c < nCols; c++) {
        const double v = GetRow(i)[c];
        a[c] += v;
        q[c] += v * v;
      }
  });
  double tr = 0.0;
  for (int c = 0; c < nCols; c++) {
    double m = 0.0, m2 = 0.0;
    for (int t = 0; t < nt; t++) m += s1[(size_t)t * nCols + c], m2 += s2[(size_t)t * nCols + c];
    m /= (double)nRows;
    tr += (m2 - (double)nRows * m * m) / (double)(nRows - 1);
  }
  return tr;
}

// --------------------------------------------------------------- mixture
GaussianMixture::GaussianMixture(int components, int cols)
    : K(components), d(cols), weights(components, 1.0 / components), means((size_t)components * cols, 0.0),
      covs((size_t)components * cols * cols, 0.0) {
  for (int j = 0; j < K; j++)
    for (int a = 0; a < d; a++) covs[((size_t)j * d + a) * d + a] = 1.0;
}

GaussianMixture GaussianMixture::Read(FILE *f) {
  int32_t k = 0, dd = 0;
  if (std::fread(&k, 4, 1, f) != 1 || std::fread(&dd, 4, 1, f) != 1 || k <= 0 || dd <= 0)
    throw FileException("invalid .cmp header");
  GaussianMixture G(k, dd);
  for (int j = 0; j < k; j++) {
    if (std::fread(G.covs.data() + (size_t)j * dd * dd, 8, (size_t)dd * dd, f) != (size_t)dd * dd ||
        std::fread(G.means.data() + (size_t)j * dd, 8, dd, f) != (size_t)dd ||
        std::fread(&G.weights[j], 8, 1, f) != 1)
      throw FileException("truncated .cmp file");
  }
  double lastLogL;
  if (std::fread(&lastLogL, 8, 1, f) != 1) throw FileException("truncated .cmp file");
  return G;
}

GaussianMixture GaussianMixture::Read(const char *fname) {
  FILE *f = std::fopen(fname, "rb");
  if (!f) throw std::invalid_argument("Cannot open file with Gaussian mixture");
  try {
    GaussianMixture G = Read(f);
    std::fclose(f);
    return G;
  } catch (...) {
    std::fclose(f);
    throw;
  }
}

void GaussianMixture::Write(FILE *f, double loglike) const {
  const int32_t k = K, dd = d;
  bool ok = std::fwrite(&k, 4, 1, f) == 1 && std::fwrite(&dd, 4, 1, f) == 1;
  for (int j = 0; j < K && ok; j++)
    ok = std::fwrite(GetCovariance(j), 8, (size_t)d * d, f) == (size_t)d * d &&
         std::fwrite(GetMean(j), 8, d, f) == (size_t)d && std::fwrite(&weights[j], 8, 1, f) == 1;
  ok = ok && std::fwrite(&loglike, 8, 1, f) == 1;
  if (!ok) throw FileException("write failed");
}

void GaussianMixture::Write(const char *fname, double loglike) const {
  FILE *f = std::fopen(fname, "wb");
  if (!f) throw FileException(std::string("cannot create ") + fname);
  try {
    Write(f, loglike);
  } catch (...) {
    std::fclose(f);
    throw;
  }
  std::fclose(f);
}

void GaussianMixture::Init(const std::vector<double> &w, const std::vector<double> &c, const std::vector<double> &m) {
  if (w.size() != (size_t)K || m.size() != (size_t)K * d || c.size() != (size_t)K * d * d)
    throw std::invalid_argument("GaussianMixture::Init: sizes do not match the mixture");
  weights = w;
  covs = c;
  means = m;
  chol.clear();
}

void GaussianMixture::Factor() const {
  if (!chol.empty()) return;
  chol.assign((size_t)K * d * d, 0.0);
  logc.assign(K, 0.0);
  for (int j = 0; j < K; j++) {
    const double *S = GetCovariance(j);
    double *L = chol.data() + (size_t)j * d * d;
    double ld = 0.0;
    for (int c = 0; c < d; c++) {
      double s = S[(size_t)c * d + c];
      for (int k = 0; k < c; k++) s -= L[(size_t)c * d + k] * L[(size_t)c * d + k];
      if (!(s > 0.0)) throw EMException("Cholesky decomposition failed");
      const double l = std::sqrt(s);
      L[(size_t)c * d + c] = l;
      ld += std::log(l);
      for (int r = c + 1; r < d; r++) {
        double t = S[(size_t)r * d + c];
        for (int k = 0; k < c; k++) t -= L[(size_t)r * d + k] * L[(size_t)c * d + k];
        L[(size_t)r * d + c] = t / l;
      }
    }
    logc[j] = std::log(weights[j]) - 0.5 * d * std::log(2.0 * M_PI) - ld;
  }
}

double GaussianMixture::LogDensities(const float *x, std::vector<double> &l) const {
  Factor();
  l.resize(K);
  std::vector<double> y(d);
  double mx = -INFINITY;
  for (int j = 0; j < K; j++) {
    const double *L = chol.data() + (size_t)j * d * d;
    const double *mu = GetMean(j);
    double q = 0.0;
    for (int r = 0; r < d; r++) {
      double t = (double)x[r] - mu[r];
      for (int k = 0; k < r; k++) t -= L[(size_t)r * d + k] * y[k];
      y[r] = t / L[(size_t)r * d + r];
      q += y[r] * y[r];
    }
    l[j] = logc[j] - 0.5 * q;
    mx = std::max(mx, l[j]);
  }
  return mx;
}

double GaussianMixture::Evaluate(const float *x) const {
  std::vector<double> l;
  const double mx = LogDensities(x, l);
  double s = 0.0;
  for (double v : l) s += std::exp(v - mx);
  return std::exp(mx) * s;
}

int GaussianMixture::Classify(const float *x) const {
  std::vector<double> l;
  LogDensities(x, l);
  int cls = 0;
  for (int j = 1; j < K; j++)
    if (l[j] > l[cls]) cls = j;
  return cls;
}

namespace {

// |lambda_max / lambda_min| of the symmetric matrix whose lower triangle is
// S (d x d, row-major): cyclic Jacobi rotations (the classical symmetric
// Schur rotation, tangent of the smaller angle) until the off-diagonal mass
// is below 1e-30 of the diagonal's, or 100 sweeps
double condition_number(const double *S, int d) {
  std::vector<double> A((size_t)d * d);
  for (int r = 0; r < d; r++)
    for (int c = 0; c < d; c++) A[(size_t)r * d + c] = c <= r ? S[(size_t)r * d + c] : S[(size_t)c * d + r];
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, dg = 0.0;
    for (int r = 0; r < d; r++)
      for (int c = 0; c < d; c++) {
        const double v = A[(size_t)r * d + c];
        if (c > r) off += v * v;
        else if (c == r) dg += v * v;
      }
    if (!(off > 1e-30 * dg)) break;
    for (int p = 0; p < d - 1; p++)
      for (int q = p + 1; q < d; q++) {
        const double apq = A[(size_t)p * d + q];
        if (apq == 0.0) continue;
        const double th = (A[(size_t)q * d + q] - A[(size_t)p * d + p]) / (2.0 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int r = 0; r < d; r++) {   // columns p, q
          const double arp = A[(size_t)r * d + p], arq = A[(size_t)r * d + q];
          A[(size_t)r * d + p] = cs * arp - sn * arq;
          A[(size_t)r * d + q] = sn * arp + cs * arq;
        }
        for (int r = 0; r < d; r++) {   // rows p, q
          const double apr = A[(size_t)p * d + r], aqr = A[(size_t)q * d + r];
          A[(size_t)p * d + r] = cs * apr - sn * aqr;
          A[(size_t)q * d + r] = sn * apr + cs * aqr;
        }
      }
  }
  double mn = A[0], mx = A[0];
  for (int p = 1; p < d; p++) mn = std::min(mn, A[(size_t)p * d + p]), mx = std::max(mx, A[(size_t)p * d + p]);
  return std::fabs(mx / mn);
}

}  // namespace

double GaussianMixture::FindLargestConditionNumber() const {
  double maxcond = 1.0;
  for (int j = 0; j < K; j++) maxcond = std::max(maxcond, condition_number(GetCovariance(j), d));
  return maxcond;
}

void GaussianMixture::Dump(FILE *f) const {
  std::fprintf(f, "Number of components: %d\n", K);
  for (int j = 0; j < K; j++) {
    std::fprintf(f, "Component %d: \n", j);
    std::fprintf(f, "Mixing probability: %g\n", weights[j]);
    std::fprintf(f, "Mean vector: ");
    for (int q = 0; q < d; q++) std::fprintf(f, "%.3g ", GetMean(j)[q]);
    std::fprintf(f, "\nCovariance matrix\n");
    for (int a = 0; a < d; a++) {
      for (int b = 0; b < d; b++) std::fprintf(f, "%.3g ", GetCovariance(j)[(size_t)a * d + b]);
      std::fprintf(f, "\n");
    }
  }
  std::fprintf(f, "Condition number of the solution: %g\n", FindLargestConditionNumber());
}

// ---------------------------------------------------------------------- EM
CudaEM::CudaEM(int ncols, int64_t nrows, int ncl, int precision, int device) : nCols(ncols), K(ncl), nRows(nrows) {
  fem_em_config cfg;
  fem_em_config_default(&cfg);
  cfg.precision = precision;
  cfg.device = device;
  check(fem_em_create(ncols, nrows, ncl, &cfg, &h));
}

CudaEM::~CudaEM() { fem_em_destroy(h); }

void CudaEM::SetParameters(int sweeps, double eps, double abortThr, double regCoef) {
  maxSweeps = sweeps;
  check(fem_em_set_parameters(h, sweeps, eps, abortThr, regCoef));
}

void CudaEM::CopyDataset(const Dataset &data) {
  if (data.GetColCount() != nCols || data.GetRowCount() != nRows)
    throw std::invalid_argument("dataset shape differs from the EM algorithm's");
  check(fem_em_upload(h, data.Data(), nCols));
}

double CudaEM::Train(const Dataset &data, GaussianMixture &G, int verbosity, bool svd) {
  CopyDataset(data);
  return TrainNoCopy(G, verbosity, svd);
}

double CudaEM::TrainNoCopy(GaussianMixture &G, int verbosity, bool svd) {
  if (G.GetComponentCount() != K || G.GetDimension() != nCols)
    throw std::invalid_argument("mixture shape differs from the EM algorithm's");
  check(fem_em_set_params(h, G.Weights().data(), G.Means().data(), G.Covs().data()));
  const int cap = std::max(1, std::min(maxSweeps, 1 << 20));
  logl.assign(cap, NAN);
  e.assign(cap, NAN);
  int iters = 0;
  double ll = NAN;
  const int st = fem_em_train(h, svd ? 1 : 0, logl.data(), e.data(), cap, &iters, &ll);
  iterCounter = iters;
  const int sweeps = std::max(0, std::min(iters - 1, cap));
  logl.resize(sweeps);
  e.resize(sweeps);
  if (verbosity > 1)
    for (int i = 0; i < sweeps; i++) std::printf("iter: %d LogL: %10.6f e: %g\n", i + 1, logl[i], e[i]);
  check(st);
  std::vector<double> w(K), m((size_t)K * nCols), c((size_t)K * nCols * nCols);
  check(fem_em_get_params(h, w.data(), m.data(), c.data()));
  G.Init(w, c, m);
  return ll;
}

void CudaEM::RetrieveClasses(std::vector<int32_t> &classes) const {
  classes.resize(nRows);
  check(fem_em_retrieve_classes(h, classes.data()));
}

void CudaEM::ComputePosterriorCorrelation(std::vector<double> &corr) const {
  corr.resize((size_t)K * K);
  check(fem_em_posterior_correlation(h, corr.data()));
}

const char *CudaEM::GetName() const { return "cudaem (GB300 tcgen05)"; }

// ---------------------------------------------------------------- k-means
CudaKMeans::CudaKMeans(const Dataset &data, int nclusters, int precision, int device, uint64_t seed, bool repair)
    : nRows(data.GetRowCount()), nCols(data.GetColCount()), K(nclusters) {
  fem_km_config cfg;
  fem_km_config_default(&cfg);
  cfg.precision = precision;
  cfg.device = device;
  cfg.seed = seed;
  cfg.repair = repair ? 1 : 0;
  check(fem_km_create(nCols, nRows, K, &cfg, &h));
  check(fem_km_upload(h, data.Data(), nCols));
}

CudaKMeans::~CudaKMeans() { fem_km_destroy(h); }

double CudaKMeans::RunKMeans(std::vector<double> &vec, int verbosity, double minRel, int maxIter) {
  if (vec.size() != (size_t)K * nCols) throw std::invalid_argument("centroid vector has the wrong size");
  double best = 0.0;
  int iters = 0;
  check(fem_km_run(h, vec.data(), minRel, maxIter, &best, &iters));
  iterCount = iters;
  if (verbosity > 0) std::printf("k-means: %d iterations, fit %.12g\n", iters, best);
  return best;
}

double CudaKMeans::ComputeMSEAndCorrect(std::vector<double> &vec) {
  double fit = 0.0;
  check(fem_km_compute_mse_and_correct(h, vec.data(), &fit, nullptr));
  iterCount++;
  return fit;
}

void CudaKMeans::InitDataStructures() { check(fem_km_init_data_structures(h)); }

void CudaKMeans::Assignment(std::vector<int32_t> &labels) const {
  labels.resize(nRows);
  check(fem_km_get_assignment(h, labels.data()));
}

void CudaKMeans::SetRngState(const std::string &state) { check(fem_km_set_rng_state(h, state.c_str())); }

std::string CudaKMeans::GetRngState() const {
  std::vector<char> buf(FEM_KM_RNG_STATE_LEN);
  check(fem_km_get_rng_state(h, buf.data(), buf.size()));
  return std::string(buf.data());
}

std::string Rand::State() const {
  std::ostringstream out;
  out << rng;
  return out.str();
}

void Rand::SetState(const std::string &state) {
  std::istringstream in(state);
  if (!(in >> rng)) throw std::invalid_argument("not an mt19937_64 state");
  uni.reset();
}

std::vector<double> Forgy(const Dataset &data, int K, Rand &rnd) {
  const int64_t N = data.GetRowCount();
  const int d = data.GetColCount();
  std::vector<double> C((size_t)K * d);
  for (int j = 0; j < K; j++) {
    const int64_t obj = (int64_t)(rnd() * (double)N);
    for (int q = 0; q < d; q++) C[(size_t)j * d + q] = data.GetRow(obj)[q];
  }
  return C;
}

// ------------------------------------------------------------ initialisers
std::vector<double> KMeansPlusPlus(const Dataset &data, int K, Rand &rnd, int64_t sample) {
  const int64_t N = data.GetRowCount();
  const int d = data.GetColCount();
  if (sample <= 0 || sample >= N) return WeightedPlusPlus(data.GetRow(0), N, d, nullptr, K, rnd);
  // `sample` rows spread evenly over the dataset
  std::vector<float> P((size_t)sample * d);
  for (int64_t s = 0; s < sample; s++)
    std::copy(data.GetRow(s * (N / sample)), data.GetRow(s * (N / sample)) + d, P.begin() + (size_t)s * d);
  return WeightedPlusPlus(P.data(), sample, d, nullptr, K, rnd);
}

std::vector<double> WeightedPlusPlus(const float *P, int64_t M, int d, const double *w, int K, Rand &rnd) {
  std::vector<double> C((size_t)K * d, 0.0), best(M, DBL_MAX), agg(M);
  const int64_t first = std::min<int64_t>(M - 1, (int64_t)(rnd() * (double)M));
  for (int q = 0; q < d; q++) C[q] = P[(size_t)first * d + q];
  for (int j = 1; j < K; j++) {
    const double *c = C.data() + (size_t)(j - 1) * d;
    parallel_rows(M, [&](int64_t b, int64_t e, int) {
      for (int64_t m = b; m < e; m++) {
        double s = 0.0;
        for (int q = 0; q < d; q++) {
          const double t = c[q] - (double)P[(size_t)m * d + q];
          s += t * t;
        }
        best[m] = std::min(best[m], s);
      }
    });
    double sum = 0.0;
    for (int64_t m = 0; m < M; m++) {
      sum += best[m] * (w ? w[m] : 1.0);
      agg[m] = sum;
    }
    for (int64_t m = 0; m < M; m++) agg[m] /= sum;
    const double r = rnd();
    for (int64_t m = 0; m < M; m++)
      if (r <= agg[m]) {
        for (int q = 0; q < d; q++) C[(size_t)j * d + q] = P[(size_t)m * d + q];
        break;
      }
  }
  return C;
}

std::vector<double> KMeansOrOr(const Dataset &data, int K, Rand &rnd, double oversample) {
  const int64_t N = data.GetRowCount();
  const int d = data.GetColCount();
  const int rounds = oversample <= 0.1 ? 10 : 5;
  std::vector<double> best(N, DBL_MAX);
  std::vector<int> owner(N, -1);
  std::vector<float> cand;   // candidate rows, C x d
  // squared distance of two float rows: per-coordinate terms in float, summed in double
  auto dist = [d](const float *a, const float *b) {
    double s = 0.0;
    for (int q = 0; q < d; q++) {
      const float t = b[q] - a[q];
      s += (double)(t * t);
    }
    return s;
  };
  auto add = [&](const std::vector<float> &nc) {
    const int base = (int)(cand.size() / d), m = (int)(nc.size() / d);
    parallel_rows(N, [&](int64_t b, int64_t e, int) {
      for (int64_t i = b; i < e; i++) {
        const float *row = data.GetRow(i);
        for (int j = 0; j < m; j++) {
          const double s = dist(&nc[(size_t)j * d], row);
          if (s < best[i]) {
            best[i] = s;
            owner[i] = base + j;
          }
        }
      }
    });
    cand.insert(cand.end(), nc.begin(), nc.end());
  };
  auto cost = [&]() {
    double s = 0.0;
    for (int64_t i = 0; i < N; i++) s += best[i];
    return s;
  };
  const int64_t first = std::min<int64_t>(N - 1, (int64_t)(rnd() * (double)N));
  add(std::vector<float>(data.GetRow(first), data.GetRow(first) + d));
  double c = cost();
  for (int r = 0; r < rounds; r++) {
    // one pass in row order, so the generator is consumed as by the reference on one thread
    std::vector<float> nc;
    for (int64_t i = 0; i < N; i++)
      if (rnd() < oversample * (double)K * best[i] / c) nc.insert(nc.end(), data.GetRow(i), data.GetRow(i) + d);
    add(nc);
    c = cost();
  }
  const int64_t M = (int64_t)(cand.size() / d);
  std::vector<double> w(M, 0.0);
  for (int64_t i = 0; i < N; i++) w[owner[i]] += 1.0;
  return WeightedPlusPlus(cand.data(), M, d, w.data(), K, rnd);
}

namespace {

// KMeansEMInitializer::Init after the seeding (EM2/EMInitializer.cpp:103-134):
// 30 k-means iterations with MinRel 1e-4 on the GPU, the classes of the final
// centroids, then the class covariances (divided by count - 1) and weights
GaussianMixture MixtureFromCentroids(const Dataset &data, std::vector<double> C, int K, Rand &rnd, int precision,
                                     int device) {
  const int64_t N = data.GetRowCount();
  const int d = data.GetColCount();
  std::vector<int32_t> lab;
  {
    const int kprec = (precision == FEM_PREC_MIXED && d == 32) ? FEM_PREC_MIXED : FEM_PREC_FP32;
    CudaKMeans km(data, K, kprec, device, 0, true);
    km.SetRngState(rnd.State());   // CentroidRandomRepair draws from the same Rand() stream
    km.RunKMeans(C, 0, 1e-4, 30);
    rnd.SetState(km.GetRngState());
    // the classes of the final centroids (ClassifyDataset): one more assignment
    std::vector<double> C2 = C;
    km.ComputeMSEAndCorrect(C2);
    km.Assignment(lab);
  }
  const int nt = host_threads();
  std::vector<double> cs((size_t)nt * K * d * d, 0.0);
  std::vector<int64_t> cnt((size_t)nt * K, 0);
  parallel_rows(N, [&](int64_t b, int64_t e, int t) {
    std::vector<double> r(d);
    for (int64_t i = b; i < e; i++) {
      const int c = lab[i];
      cnt[(size_t)t * K + c]++;
      for (int q = 0; q < d; q++) r[q] = (double)data.GetRow(i)[q] - C[(size_t)c * d + q];
      double *S = cs.data() + ((size_t)t * K + c) * d * d;
      for (int a = 0; a < d; a++)
        for (int q = 0; q < d; q++) S[(size_t)a * d + q] += r[a] * r[q];
    }
  });
  GaussianMixture G(K, d);
  for (int j = 0; j < K; j++) {
    int64_t n = 0;
    for (int t = 0; t < nt; t++) n += cnt[(size_t)t * K + j];
    for (size_t e = 0; e < (size_t)d * d; e++) {
      double s = 0.0;
      for (int t = 0; t < nt; t++) s += cs[((size_t)t * K + j) * d * d + e];
      G.Covs()[(size_t)j * d * d + e] = s / ((double)n - 1.0);
    }
    for (int q = 0; q < d; q++) G.Means()[(size_t)j * d + q] = C[(size_t)j * d + q];
    G.Weights()[j] = (double)n / (double)N;
  }
  return G;
}

}  // namespace

GaussianMixture InitMixture(const char *name, const Dataset &data, int K, Rand &rnd, int precision, int device) {
  const int64_t N = data.GetRowCount();
  const int d = data.GetColCount();
  if (name == nullptr || !std::strcmp(name, "jain")) {
    // JainEMInitializer::Init (EM2/EMInitializer.cpp:43-77): means are rows
    // at Rand() * N, covariances tr(Cov) / d / 10 I, weights 1 / K.  The
    // reference draws a component's row once, then keeps drawing until a
    // draw misses the rows already taken, but keeps the first draw (the
    // repeat test reads a shadowing variable): the same rows and the same
    // use of the stream here, repeats included.
    // Once the rows taken cover all N rows no draw can miss them: the
    // reference loops forever there (K > N); here the redraws stop.
    GaussianMixture G(K, d);
    const double cv = data.GetCovMatrixTrace() / d / 10.0;
    std::unordered_set<int64_t> taken;
    for (int j = 0; j < K; j++) {
      const int64_t idx = (int64_t)(rnd() * (double)N);
      while ((int64_t)taken.size() < N) {
        const int64_t again = (int64_t)(rnd() * (double)N);
        if (!taken.count(again)) break;
      }
      taken.insert(idx);
      for (int q = 0; q < d; q++) G.Means()[(size_t)j * d + q] = data.GetRow(idx)[q];
      for (int a = 0; a < d; a++)
        for (int b = 0; b < d; b++) G.Covs()[((size_t)j * d + a) * d + b] = a == b ? cv : 0.0;
      G.Weights()[j] = 1.0 / K;
    }
    return G;
  }
  if (!std::strcmp(name, "kmeans")) {
    // KMeansEMInitializer (EM2/EMInitializer.cpp:80-134): Forgy centroids,
    // then k-means and class covariances
    return MixtureFromCentroids(data, Forgy(data, K, rnd), K, rnd, precision, device);
  }
  if (!std::strcmp(name, "kmeansoror")) {
    // KMeansOrOrEMInitializer (EM2/EMInitializer.cpp:153-157): k-means||
    // centroids with oversampling 1.4, then as above
    return MixtureFromCentroids(data, KMeansOrOr(data, K, rnd, 1.4), K, rnd, precision, device);
  }
  return GaussianMixture::Read(name);
}

}  // namespace fastem
