/*
 * eg_oracle.h — CPU restatement of EndGraph's preprocessing and Gemini's process_edges
 * toolkits, used ONLY as a test checker (tests/, __graft_entry__.smoke(), bench.py's
 * cpu_baseline leg).  The product never links or calls this code.
 *
 * Every function cites the reference lines it restates (paths inside leodestiny/EndGraph).
 * Parity of this restatement is pinned against the reference's own engine compiled at one rank
 * (oracle/build_ref.sh -> oracle/_ref/libeg_ref.so) and against committed golden vectors.
 */
#ifndef EG_ORACLE_H
#define EG_ORACLE_H

#include <stdint.h>
#include "../include/endgraph_rmat.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORA_PAGESIZE 4096u /* core/constants.hpp:21 */
#define ORA_UNREACHED 0xFFFFFFFFu

/* Generate edges [e0, e0+n) of an R-MAT stream (input definition, not reference code). */
void ora_rmat(const eg_rmat_params* p, uint64_t e0, uint64_t n, uint32_t* src, uint32_t* dst, float* w);

/* Degree histogram, core/graph.hpp:689-707 (both directions in one pass). */
void ora_degrees(const uint32_t* src, const uint32_t* dst, uint64_t E, uint32_t V,
                 uint32_t* outdeg, uint32_t* indeg);

/* CPBT page weights, core/graph.hpp:718-741. */
void ora_page_weights(const uint32_t* deg, uint32_t V, int P, uint64_t eta, int max_iterations,
                      int dense, uint64_t* page_amount);

/* optimal_offset + judge, core/graph.hpp:586-626. offset has k+1 entries. */
void ora_optimal_offset(const uint64_t* a, uint32_t n, uint32_t k, uint32_t* offset);

/* assign_vertices boundaries for P partitions and S sub-partitions each,
 * core/graph.hpp:743-749 and :774-780 (the latter evaluated for every partition).
 * partition_offset: P+1; local_offset: P*(S+1). */
void ora_cpbt(const uint32_t* deg, uint32_t V, int P, int S, uint64_t eta, int max_iterations,
              int dense, uint32_t* partition_offset, uint32_t* local_offset);

/* Owner of vertex v under (possibly non-monotone) offsets: first i with off[i] <= v < off[i+1],
 * core/graph.hpp:404-412. */
int ora_partition_of(const uint32_t* partition_offset, int P, uint32_t v);

/* Push structure, prepare_push_mode core/graph.hpp:1248-1355 with the P-way owner split of
 * shuffle_edge_list (key dst) core/graph.hpp:988-992.  Partition p holds the edges whose dst it
 * owns, stably sorted by src (file order inside a list).  Positions are absolute (partitions are
 * concatenated); part_start[P+1]; csr_off[P*(V+1)] dense; bitmap[P*nwords] (nwords = V/64+1).
 * csr_w may be NULL. */
void ora_build_csr(const uint32_t* src, const uint32_t* dst, const float* w, uint64_t E, uint32_t V,
                   int P, const uint32_t* partition_offset, uint64_t* part_start, uint64_t* csr_off,
                   uint32_t* csr_dst, float* csr_w, uint64_t* bitmap);

/* Pull structure, prepare_pull_mode core/graph.hpp:1098-1188 (shuffle key src, :999-1003).
 * Partition p holds the edges whose src it owns, sorted by dst; inside a dst list the order is
 * ascending src (ties in file order), which is what the reference produces when the push
 * structure is built first (its in-place sort by src precedes the sort by dst).
 * csc_off dense [P*(V+1)]; compressed index per partition: entries (vertex, absolute index) for
 * each distinct dst plus a sentinel (V, part end); cstart[P+1] gives entry ranges.
 * Returns the total number of compressed entries (including sentinels).  ccap = capacity. */
uint64_t ora_build_csc(const uint32_t* src, const uint32_t* dst, const float* w, uint64_t E, uint32_t V,
                       int P, const uint32_t* partition_offset, uint64_t* part_start, uint64_t* csc_off,
                       uint32_t* csc_src, float* csc_w, uint64_t* cstart, uint32_t* cvert, uint64_t* cidx,
                       uint64_t ccap);

/* Gemini PageRank, toolkits/pagerank.cpp:26-98, dense mode, double precision, sums taken in CSC
 * list order.  out[V]. */
void ora_pagerank(const uint64_t* csc_off, const uint32_t* csc_src, const uint32_t* outdeg,
                  uint32_t V, int iterations, double damping, double* out);

/* BFS levels from root, toolkits/bfs.cpp:22-84 (level = iteration that first activates v). */
void ora_bfs_levels(const uint64_t* csr_off, const uint32_t* csr_dst, uint32_t V, uint32_t root,
                    uint32_t* level);

/* Count BFS-tree violations of parent[] given exact levels (parent == V: unreached). */
uint64_t ora_bfs_check_parents(const uint64_t* csr_off, const uint32_t* csr_dst, uint32_t V,
                               uint32_t root, const uint32_t* level, const uint32_t* parent);

/* Connected-component labels (min vertex id of each component of the symmetrised graph),
 * the fixpoint of toolkits/cc.cpp:22-84 on load_undirected_from_directed input. */
void ora_cc_labels(const uint32_t* src, const uint32_t* dst, uint64_t E, uint32_t V, uint32_t* label);

/* SSSP distances (float, sentinel 1e9), the least fixpoint of toolkits/sssp.cpp:24-84. */
void ora_sssp(const uint64_t* csr_off, const uint32_t* csr_dst, const float* csr_w, uint32_t V,
              uint32_t root, float* dist);

/* Single-source betweenness dependencies (Brandes 2001; BC is named by the reference README,
 * README.md:24,37, without code in its tree): BFS over out-edges counting shortest paths sigma,
 * then delta[v] = sum over out-neighbours w one level deeper of sigma[v]/sigma[w]*(1+delta[w]),
 * accumulated in reverse BFS order.  level: BFS level, ORA_UNREACHED when unreached. */
void ora_bc(const uint64_t* csr_off, const uint32_t* csr_dst, uint32_t V, uint32_t root, double* sigma,
            double* delta, uint32_t* level);

/* Order-independent per-vertex neighbour signatures: hout[s] += mix(d | wbits<<32),
 * hin[d] += mix(s | wbits<<32) (wbits = 0 when w is NULL). */
void ora_adjacency_hash(const uint32_t* src, const uint32_t* dst, const float* w, uint64_t E, uint32_t V,
                        uint64_t* hout, uint64_t* hin);

/* The same signature per list of a CSR/CSC: h[v] = sum over [off[v], off[v+1]) of
 * mix(adj[e] | wbits<<32), so h equals hout (CSR) or hin (CSC) of the edge list it was built from,
 * whatever the order inside each list. */
void ora_list_hash(const uint64_t* off, const uint32_t* adj, const float* w, uint64_t n, uint64_t* h);

#ifdef __cplusplus
}
#endif
#endif
