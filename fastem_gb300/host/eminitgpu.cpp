// eminitgpu -- the reference's eminit (EM2/eminit.cpp): builds the initial
// mixture of a dataset with one of the EM initialisers and writes it as a
// .cmp file (-o) or prints it (GaussianMixture::Dump).  Same options:
//
//   eminitgpu file.bin [-c components] [-I init] [-r seed] [-o mixture.cmp]
//             [-p mixed|fp32|fp64] [-d device]
//
// init (-I): kmeans (default), kmeansoror, jain, or a .cmp file
// (CreateEMInitializer, EM2/EMInitializer.cpp:168-177).  The k-means
// initialisers run their 30 k-means iterations on the GPU (-p picks the
// k-means precision: mixed takes the tensor-core assignment when d = 32,
// FP32 CUDA cores otherwise); jain and file need no GPU.
// A bad option prints "Invalid program argument: ..." as eminit does, and
// exits with status 1.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <unistd.h>

#include "fastem.hpp"

using namespace fastem;

namespace {

struct Args {
  int ncl = 1, seed = 0, precision = FEM_PREC_MIXED, device = 0;
  const char *iname = "kmeans", *oname = nullptr, *fname = nullptr;
};

// ProcessArgs (EM2/eminit.cpp): -o -I -r -c, then the dataset name
Args process_args(int argc, char *argv[]) {
  Args a;
  int c;
  while ((c = getopt(argc, argv, "o:I:r:c:p:d:")) != -1) {
    switch (c) {
      case 'o': a.oname = optarg; break;
      case 'I': a.iname = optarg; break;
      case 'r':
        a.seed = std::atoi(optarg);
        if (a.seed < 0) throw std::invalid_argument("invalid value of -r option");
        break;
      case 'c':
        a.ncl = std::atoi(optarg);
        if (a.ncl <= 0) throw std::invalid_argument("invalid value of -c option");
        break;
      case 'p':
        if (!std::strcmp(optarg, "mixed")) a.precision = FEM_PREC_MIXED;
        else if (!std::strcmp(optarg, "fp32")) a.precision = FEM_PREC_FP32;
        else if (!std::strcmp(optarg, "fp64")) a.precision = FEM_PREC_FP64;
        else throw std::invalid_argument("invalid value of -p option");
        break;
      case 'd': a.device = std::atoi(optarg); break;
      default: throw std::invalid_argument("Invalid command line option");
    }
  }
  if (optind >= argc) throw std::invalid_argument("Missing dataset name");
  a.fname = argv[optind];
  return a;
}

const char *init_info(const char *name) {
  if (!std::strcmp(name, "jain")) return "Jain EM Initializer";
  if (!std::strcmp(name, "kmeans")) return "K-means EM initializer";
  if (!std::strcmp(name, "kmeansoror")) return "K-means|| EM initializer";
  return "File EM initializer";
}

}  // namespace

int main(int argc, char *argv[]) {
  Args a;
  try {
    a = process_args(argc, argv);
  } catch (std::invalid_argument &e) {
    std::printf("Invalid program argument: %s\n", e.what());
    return 1;
  }
  try {
    std::printf("Seed of rng: %d\n", a.seed);
    Rand rnd((unsigned)a.seed);
    std::printf("Loading dataset %s... ", a.fname);
    Dataset D = Dataset::Load(a.fname);
    std::printf("%lld vectors, %d features\n", (long long)D.GetRowCount(), D.GetColCount());
    std::printf("Covariance matrix trace: %10.10g\n", D.GetCovMatrixTrace());
    std::printf("Number of components: %d\n", a.ncl);
    std::printf("%s\n", init_info(a.iname));
    GaussianMixture G = InitMixture(a.iname, D, a.ncl, rnd, a.precision, a.device);
    if (a.oname) G.Write(a.oname);
    else G.Dump();
  } catch (std::exception &e) {
    std::fprintf(stderr, "eminitgpu: %s\n", e.what());
    return 1;
  }
  return 0;
}
