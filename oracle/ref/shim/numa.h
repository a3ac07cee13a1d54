/*
 * One-node libnuma stand-in used only to compile the reference sources into the oracle.
 * numa_num_configured_cpus() returns zgref_num_cpus (1 unless a driver sets it), so
 * SharedMemSys (src/SharedMemSys.cpp:17-22) runs the estimators on one thread for replay.
 * Allocations are zero-filled, like the fresh pages numa_alloc_onnode maps.
 * Test infrastructure, not product code.
 */
#ifndef ZGREF_SHIM_NUMA_H
#define ZGREF_SHIM_NUMA_H

#include <stdlib.h>

struct bitmask { unsigned long size; unsigned long* maskp; };

extern int zgref_num_cpus;

static inline int numa_available(void) { return 0; }
static inline int numa_num_configured_cpus(void) { return zgref_num_cpus; }
static inline int numa_num_configured_nodes(void) { return 1; }
static inline struct bitmask* numa_parse_nodestring(const char*) {
  static struct bitmask b = {0, 0};
  return &b;
}
static inline void numa_set_interleave_mask(struct bitmask*) {}
static inline int numa_run_on_node(int) { return 0; }
static inline void* numa_alloc_onnode(size_t size, int) { return calloc(size ? size : 1, 1); }
static inline void* numa_alloc_interleaved(size_t size) { return calloc(size ? size : 1, 1); }
static inline void numa_free(void* p, size_t) { free(p); }

#endif
