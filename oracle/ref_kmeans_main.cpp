// Driver for the reference's own k-means (NaiveKMA, Clust/KMAlgorithm.cpp,
// with CentroidVector, OpenMPKMAReducer and CentroidRandomRepair, compiled in
// place by `make -C oracle ref`; test infrastructure only).
//
//   ref_kmeans data.bin centroids.f64 iterations seed out.bin
//
// Loads the dataset with MultithreadedDataset::Load, reads k x d FP64
// centroids, seeds the reference's generator (SRand, used by the random
// repair), and runs `iterations` NaiveKMA::ComputeMSEAndCorrect calls.  Before
// each call the labels of the current centroids are taken with
// CentroidVector::ClassifyDataset.  out.bin: int32 iterations, n, k, d; then
// per iteration the fit (FP64), n int32 labels, k x d FP64 centroids after the
// update.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "Clust/CentroidRepair.h"
#include "Clust/CentroidVector.h"
#include "Clust/KMAlgorithm.h"
#include "Util/MultithreadedDataset.h"
#include "Util/NumaAlloc.h"
#include "Util/Rand.h"

int main(int argc, char *argv[]) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: ref_kmeans data.bin centroids.f64 iterations seed out.bin\n");
    return 1;
  }
  const int iters = std::atoi(argv[3]);
  SRand((unsigned)std::strtoul(argv[4], nullptr, 10));
  NUMAAllocator::CreateNUMAAllocator();
  MultithreadedDataset D;
  D.Load(argv[1]);
  const long n = D.GetRowCount();
  const int d = D.GetColCount();
  FILE *fc = std::fopen(argv[2], "rb");
  if (!fc) return 2;
  std::vector<double> c;
  double v;
  while (std::fread(&v, sizeof v, 1, fc) == 1) c.push_back(v);
  std::fclose(fc);
  if (c.empty() || c.size() % d) return 3;
  const int k = (int)(c.size() / d);
  DynamicArray<OPTFLOAT> vec(k * d);
  for (int i = 0; i < k * d; i++) vec[i] = c[i];
  CentroidVector CV(k, d);
  CentroidRandomRepair repair(D, k);
  NaiveKMA alg(CV, D, &repair);
  alg.InitDataStructures(vec);
  DynamicArray<int> labels(n);
  FILE *fo = std::fopen(argv[5], "wb");
  if (!fo) return 4;
  const int hdr[4] = {iters, (int)n, k, d};
  std::fwrite(hdr, sizeof(int), 4, fo);
  for (int it = 0; it < iters; it++) {
    CV.ClassifyDataset(vec, D, labels);
    const double fit = alg.ComputeMSEAndCorrect(vec);
    std::fwrite(&fit, sizeof fit, 1, fo);
    for (long i = 0; i < n; i++) {
      const int l = labels[i];
      std::fwrite(&l, sizeof l, 1, fo);
    }
    for (int i = 0; i < k * d; i++) {
      const double x = vec[i];
      std::fwrite(&x, sizeof x, 1, fo);
    }
  }
  std::fclose(fo);
  return 0;
}
