// Driver for the reference's own generator (Util/Rand.cpp, compiled in place
// by `make -C oracle ref`; test infrastructure only): prints `count` values of
// Rand() after SRand(seed), then `count` values of RandInt(n), one per line,
// so the oracle's restatement of the stream can be checked against it.
#include <cstdio>
#include <cstdlib>

#include "Rand.h"

int main(int argc, char *argv[]) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: ref_rand seed count n\n");
    return 1;
  }
  const unsigned seed = (unsigned)std::strtoul(argv[1], nullptr, 10);
  const long count = std::atol(argv[2]);
  const unsigned long n = std::strtoul(argv[3], nullptr, 10);
  SRand(seed);
  for (long i = 0; i < count; i++) std::printf("%.17g\n", Rand());
  for (long i = 0; i < count; i++) std::printf("%d\n", RandInt(n));
  return 0;
}
