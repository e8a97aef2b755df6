// Stand-in for libnuma's <numa.h>, for compiling the reference's k-means
// sources in place (test infrastructure only).  One NUMA node, memory where
// the first touch puts it: the three calls the reference makes
// (Util/NumaAlloc.cpp:43,81,95, Util/NumaAlloc.h:88-146) answer as libnuma
// does on a one-node machine.  No arithmetic of the path goes through them.
#pragma once

static inline int numa_num_configured_nodes(void) { return 1; }
static inline int numa_node_of_cpu(int cpu) {
  (void)cpu;
  return 0;
}
static inline void numa_tonode_memory(void *start, unsigned long size, int node) {
  (void)start;
  (void)size;
  (void)node;
}
