// em2gpu -- the reference's em2 driver (EM2/main.cpp, EM2/EMArgs.cpp) on one
// GB300.  Same options where they apply:
//
//   em2gpu file.bin [-c components] [-I init] [-r seed] [-m maxiter] [-b burnin]
//          [-f eps] [-a abort] [-g regcoeff] [-S] [-v verbosity]
//          [-o mixture.cmp] [-O classes.bin] [-p mixed|fp32|fp64] [-d device]
//   em2gpu --info file     (header and checksum of a .bin or .cmp file; no GPU)
//   em2gpu --seed pp|oror file.bin K seed   (k-means++ / k-means|| centroids; no GPU)
//
// init (-I): jain (default), kmeans, kmeansoror, or a .cmp file (EM2/EMInitializer.cpp:168-177).
// -o writes the fitted mixture (.cmp), -O the classes of every row under the
// fitted mixture, 1-based, after an int32 row count (GaussianMixture::WriteClasses).
#include <chrono>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unistd.h>

#include "fastem.hpp"

using namespace fastem;

namespace {

void usage() {
  std::printf(
      "Arguments: filename - name of the file in .bin format\n"
      "-c components : number of Gaussian mixture components\n"
      "-I init : jain, kmeans, kmeansoror or a .cmp file with the initial mixture\n"
      "-r seed : seed of the pseudo-random number generator\n"
      "-m emiter : maximal number of EM iterations\n"
      "-b burnin : number of burn-in EM iterations (default 0)\n"
      "-f eps : EM stopping threshold (default 1e-5)\n"
      "-a abort : EM failure threshold on the condition number (default 1e5)\n"
      "-g coeff : covariance regularisation coefficient (default 0)\n"
      "-S : disables the condition-number check\n"
      "-v verbosity\n"
      "-o file : writes the fitted mixture (.cmp)\n"
      "-O file : writes the classes of every row (int32 count, then 1-based classes)\n"
      "-p precision : mixed (default), fp32 or fp64\n"
      "-d device : CUDA device\n"
      "-A/-R/-M/-N/-T/-t/-u/-U : the reference's CPU tuning options, accepted and ignored\n"
      "--info file : prints the header and a checksum of a .bin or .cmp file\n"
      "--seed pp|oror file K seed : prints k-means++ / k-means|| centroids of a .bin file\n");
}

int info(const char *fname) {
  const std::string s(fname);
  if (s.size() > 4 && s.substr(s.size() - 4) == ".cmp") {
    GaussianMixture G = GaussianMixture::Read(fname);
    double sw = 0, sm = 0, sc = 0;
    for (double w : G.Weights()) sw += w;
    for (double m : G.Means()) sm += m;
    for (double c : G.Covs()) sc += c;
    std::printf("cmp components=%d dims=%d sum_weights=%.17g sum_means=%.17g sum_covs=%.17g\n",
                G.GetComponentCount(), G.GetDimension(), sw, sm, sc);
    return 0;
  }
  Dataset D = Dataset::Load(fname);
  double sum = 0.0;
  for (int64_t i = 0; i < D.GetRowCount(); i++)
    for (int c = 0; c < D.GetColCount(); c++) sum += D.GetRow(i)[c];
  std::printf("bin rows=%lld cols=%d sum=%.17g trace=%.17g\n", (long long)D.GetRowCount(), D.GetColCount(), sum,
              D.GetCovMatrixTrace());
  return 0;
}

// a refused option value: em2's message (EM2/main.cpp prints it after
// "Invalid program argument: "), exit status 1
int bad_argument(const char *msg) {
  std::printf("Invalid program argument: %s\n", msg);
  return 1;
}

}  // namespace

// the seeders on the host (no GPU): K rows of %.17g coordinates
static int seed_centroids(const char *how, const char *fname, int K, unsigned seed) {
  Dataset D = Dataset::Load(fname);
  Rand rnd(seed);
  std::vector<double> C;
  if (!std::strcmp(how, "pp")) C = KMeansPlusPlus(D, K, rnd, 0);
  else if (!std::strcmp(how, "oror")) C = KMeansOrOr(D, K, rnd, 1.4);
  else throw std::invalid_argument("--seed takes pp or oror");
  const int d = D.GetColCount();
  for (int j = 0; j < K; j++) {
    for (int q = 0; q < d; q++) std::printf(q ? " %.17g" : "%.17g", C[(size_t)j * d + q]);
    std::printf("\n");
  }
  return 0;
}

int main(int argc, char *argv[]) {
  if (argc >= 6 && !std::strcmp(argv[1], "--seed")) {
    try {
      return seed_centroids(argv[2], argv[3], std::atoi(argv[4]), (unsigned)std::strtoul(argv[5], nullptr, 10));
    } catch (std::exception &e) {
      std::fprintf(stderr, "%s\n", e.what());
      return 1;
    }
  }
  if (argc >= 3 && !std::strcmp(argv[1], "--info")) {
    try {
      return info(argv[2]);
    } catch (std::exception &e) {
      std::fprintf(stderr, "%s\n", e.what());
      return 1;
    }
  }
  int ncl = 1, maxiter = 1000000, burnin = 0, verbosity = 1, device = 0, precision = FEM_PREC_MIXED;
  unsigned seed = 0;
  double eps = 1e-5, athr = 1e5, reg = 0.0;
  bool svd = true;
  const char *iname = nullptr, *oname = nullptr, *cname = nullptr;
  int c;
  while ((c = getopt(argc, argv, "c:I:r:m:b:f:a:g:Sv:o:O:p:d:hBN:M:A:R:T:t:u:U:")) != -1) {
    switch (c) {
      // the reference's CPU tuning options (EM2/EMArgs.cpp:76-158): accepted so
      // that em2 command lines run unchanged; they select OpenMP loop shapes,
      // reducers and NUMA placement, which the GPU backend does not have
      case 'N': {
        // BlockManagerBase::ParseEMBlockParams (EM2/BlockManager.cpp:18-28)
        double l3;
        int a, b;
        if (std::sscanf(optarg, "automax:%lf", &l3) != 1 && std::sscanf(optarg, "%d:%d", &a, &b) != 2) {
          std::fprintf(stderr, "Bad value of MStepLoopParam\n");
          return 1;
        }
        break;
      }
      case 'A':
        // CreateEMAlgorithm's names (EM2/EMAlgorithm.cpp:247-269): all run on this backend
        if (std::strcmp(optarg, "matrixem") && std::strcmp(optarg, "simplematrixem") &&
            std::strcmp(optarg, "cachedem")) {
          std::fprintf(stderr, "Invalid EM algorithm name %s\n", optarg);
          return 1;
        }
        break;
      case 'M': case 'R': case 'T': case 't': case 'u': case 'U': break;
      case 'B':
        std::printf("-B benchmarks the reference's OpenMP reduction; the GPU backend has none\n");
        return 0;
      // value checks and messages of ProcessArgs (EM2/EMArgs.cpp:75-170)
      case 'c':
        if ((ncl = std::atoi(optarg)) <= 0) return bad_argument("invalid value of -c option");
        break;
      case 'I': iname = optarg; break;
      case 'r': {
        const int r = std::atoi(optarg);
        if (r < 0) return bad_argument("invalid value of -r option");
        seed = (unsigned)r;
        break;
      }
      case 'm':
        if ((maxiter = std::atoi(optarg)) < 0) return bad_argument("invalid value of -m option");
        break;
      case 'b':
        if ((burnin = std::atoi(optarg)) < 0) return bad_argument("invalid value of -b option");
        break;
      case 'f':
        if ((eps = std::atof(optarg)) <= 0.0) return bad_argument("argument to -f must be greater or than 0");
        break;
      case 'a':
        if ((athr = std::atof(optarg)) < 1.0) return bad_argument("argument to -a must be greater then 1.0");
        break;
      case 'g':
        reg = std::atof(optarg);
        if (reg < 0.0 || reg > 1.0) return bad_argument("argument to -g must be small positive number");
        break;
      case 'S': svd = false; break;
      case 'v':
        if ((verbosity = std::atoi(optarg)) < 0) return bad_argument("invalid value of -v option");
        break;
      case 'o': oname = optarg; break;
      case 'O': cname = optarg; break;
      case 'd': device = std::atoi(optarg); break;
      case 'p':
        if (!std::strcmp(optarg, "mixed")) precision = FEM_PREC_MIXED;
        else if (!std::strcmp(optarg, "fp32")) precision = FEM_PREC_FP32;
        else if (!std::strcmp(optarg, "fp64")) precision = FEM_PREC_FP64;
        else {
          usage();
          return 1;
        }
        break;
      default:
        usage();
        return 1;
    }
  }
  if (optind >= argc) {
    usage();
    return 1;
  }
  const char *fname = argv[optind];
  using clk = std::chrono::steady_clock;
  try {
    std::printf("Loading dataset %s... ", fname);
    auto t0 = clk::now();
    Dataset D = Dataset::Load(fname);
    std::printf("%lld vectors, %d features\n", (long long)D.GetRowCount(), D.GetColCount());
    std::printf("Loading took %g seconds\n", std::chrono::duration<double>(clk::now() - t0).count());
    std::printf("Covariance matrix trace: %10.10g\n", D.GetCovMatrixTrace());
    std::printf("Number of components: %d\n", ncl);
    std::printf("Regularization factor: %g\n", reg);
    std::printf("EM convergence threshold: %g\n", eps);
    std::printf("EM abort threshold: %g\n", athr);
    Rand rnd(seed);
    GaussianMixture G = InitMixture(iname, D, ncl, rnd, precision, device);
    if (G.GetComponentCount() != ncl || G.GetDimension() != D.GetColCount()) {
      // a .cmp initial mixture must match -c and the dataset (the reference
      // would read past the mixture in DecodeMixture)
      std::fprintf(stderr, "em2gpu: the initial mixture has %d components of dimension %d; -c %d on %d columns\n",
                   G.GetComponentCount(), G.GetDimension(), ncl, D.GetColCount());
      return 1;
    }
    CudaEM A(D.GetColCount(), D.GetRowCount(), ncl, precision, device);
    std::printf("Using EM algorithm %s\n", A.GetName());
    double LogL = 0.0;
    double extime = 0.0;
    try {
      A.CopyDataset(D);
      if (burnin > 0) {
        std::printf("Running %d burn-in iterations\n", burnin);
        A.SetParameters(burnin, eps, athr, reg);
        GaussianMixture G2 = G;
        t0 = clk::now();
        A.TrainNoCopy(G2, verbosity, svd);
        const double bt = std::chrono::duration<double>(clk::now() - t0).count();
        std::printf("Burn-in time: %g seconds\n", bt);
        std::printf("Burn-in iter time: %g miliseconds\n", 1000.0 * bt / std::max(1, A.GetIterCounter() - 1));
      }
      A.SetParameters(maxiter, eps, athr, reg);
      t0 = clk::now();
      LogL = A.TrainNoCopy(G, verbosity, svd);
      if (verbosity > 3) G.Dump();   // EM2/main.cpp: the fitted mixture
    } catch (EMException &e) {
      std::printf("EM algorithm failed: %s\n", e.what());
    }
    extime = std::chrono::duration<double>(clk::now() - t0).count();
    const int iters = A.GetIterCounter() - 1;
    std::printf("EM Execution time: %g seconds\n", extime);
    std::printf("%d total EM sweeps\n", iters);
    std::printf("Iteration time: %g miliseconds\n", 1000.0 * extime / std::max(1, iters));
    std::printf("Final loglikelihood: %.17g\n", LogL);
    if (oname) G.Write(oname, LogL);
    if (cname) {
      FILE *f = std::fopen(cname, "wb");
      if (!f) throw FileException(std::string("cannot create ") + cname);
      // an int32 count, or -1 and an int64 count above 2^31 - 1 rows (the
      // two forms ReadAssignment reads, Util/MultithreadedDataset.cpp:371-386)
      const int64_t rows = D.GetRowCount();
      const int32_t n32 = rows > INT32_MAX ? -1 : (int32_t)rows;
      std::vector<int32_t> cls(rows);
      for (int64_t i = 0; i < rows; i++) cls[i] = G.Classify(D.GetRow(i)) + 1;
      bool ok = std::fwrite(&n32, 4, 1, f) == 1 && (n32 != -1 || std::fwrite(&rows, 8, 1, f) == 1);
      ok = ok && std::fwrite(cls.data(), 4, cls.size(), f) == cls.size();
      std::fclose(f);
      if (!ok) throw FileException("write failed");
    }
  } catch (std::exception &e) {
    std::fprintf(stderr, "em2gpu: %s\n", e.what());
    return 1;
  }
  return 0;
}
