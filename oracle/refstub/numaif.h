// Stand-in for libnuma's <numaif.h> (see numa.h beside it): page-node queries
// (Util/NumaAlloc.h:76, Util/Array.cpp:19) report node 0 for every page.
#pragma once

static inline long move_pages(int pid, unsigned long count, void **pages, const int *nodes, int *status,
                              int flags) {
  (void)pid;
  (void)pages;
  (void)nodes;
  (void)flags;
  for (unsigned long i = 0; i < count; i++) status[i] = 0;
  return 0;
}
static inline long numa_move_pages(int pid, unsigned long count, void **pages, const int *nodes, int *status,
                                   int flags) {
  return move_pages(pid, count, pages, nodes, status, flags);
}
