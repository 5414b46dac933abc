/*
 * Single-node stand-in for <numa.h>, written for building the reference's engine as a test
 * oracle.  One NUMA node holding every CPU (EG_REF_THREADS overrides the CPU count); all
 * allocations are anonymous mmaps, zero-filled like libnuma's, released with munmap because the
 * reference frees mmap'ed vertex arrays with numa_free (core/graph.hpp:299,313).
 */
#ifndef EG_REF_NUMA_SHIM_H
#define EG_REF_NUMA_SHIM_H

#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <omp.h>

struct bitmask { unsigned long size; unsigned long* maskp; };

static inline int numa_available() { return 0; }
static inline int numa_num_configured_cpus() {
    const char* s = getenv("EG_REF_THREADS");
    if (s && atoi(s) > 0) return atoi(s);
    return omp_get_num_procs();
}
static inline int numa_num_configured_nodes() { return 1; }
static inline struct bitmask* numa_parse_nodestring(const char*) {
    static unsigned long word = 1;
    static struct bitmask m = {1, &word};
    return &m;
}
static inline void numa_set_interleave_mask(struct bitmask*) {}
static inline int numa_run_on_node(int) { return 0; }
static inline void numa_tonode_memory(void*, size_t, int) {}
static inline void* eg_numa_map_(size_t size) {
    void* p = mmap(NULL, size ? size : 1, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    return p == MAP_FAILED ? NULL : p;
}
static inline void* numa_alloc_onnode(size_t size, int) { return eg_numa_map_(size); }
static inline void* numa_alloc_interleaved(size_t size) { return eg_numa_map_(size); }
static inline void numa_free(void* p, size_t size) { if (p) munmap(p, size ? size : 1); }
static inline void* numa_realloc(void* old, size_t old_size, size_t new_size) {
    void* p = eg_numa_map_(new_size);
    if (p && old) {
        memcpy(p, old, old_size < new_size ? old_size : new_size);
        numa_free(old, old_size);
    }
    return p;
}

#endif
