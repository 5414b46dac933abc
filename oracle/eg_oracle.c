/*
 * eg_oracle.c — CPU restatement used as the test checker.  See eg_oracle.h.
 * Plain C, single-threaded except for the generator; sized for seconds-long runs.
 */
#include "eg_oracle.h"

#include <stdlib.h>
#include <string.h>

void ora_rmat(const eg_rmat_params* p, uint64_t e0, uint64_t n, uint32_t* src, uint32_t* dst, float* w) {
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < (int64_t)n; ++k) {
        float wt = 0.f;
        eg_rmat_edge(p, e0 + (uint64_t)k, &src[k], &dst[k], w ? &wt : NULL);
        if (w) w[k] = wt;
    }
}

/* core/graph.hpp:689-707: deg[dst]++ when sparse, deg[src]++ when dense; here both at once. */
void ora_degrees(const uint32_t* src, const uint32_t* dst, uint64_t E, uint32_t V,
                 uint32_t* outdeg, uint32_t* indeg) {
    memset(outdeg, 0, sizeof(uint32_t) * V);
    memset(indeg, 0, sizeof(uint32_t) * V);
    for (uint64_t i = 0; i < E; ++i) {
        outdeg[src[i]]++;
        indeg[dst[i]]++;
    }
}

/* core/graph.hpp:718-741.  The reference evaluates
 *   (1 + (P-1)/16) * degree            -> int * UINT: 32-bit unsigned arithmetic
 *   eta * (P - 1 + T * degree)          -> size_t * (32-bit unsigned)
 * with T = max_iterations when dense, 1 when sparse (:733-738), summed into a u64 per page. */
void ora_page_weights(const uint32_t* deg, uint32_t V, int P, uint64_t eta, int max_iterations,
                      int dense, uint64_t* page_amount) {
    uint32_t pages = (V + ORA_PAGESIZE - 1) / ORA_PAGESIZE;
    uint32_t c1 = (uint32_t)(1 + (P - 1) / 16);
    uint32_t T = dense ? (uint32_t)max_iterations : 1u;
    for (uint32_t i = 0; i < pages; ++i) {
        uint64_t acc = 0;
        uint32_t vb = i * ORA_PAGESIZE;
        uint32_t ve = vb + ORA_PAGESIZE < V ? vb + ORA_PAGESIZE : V;
        for (uint32_t v = vb; v < ve; ++v) {
            uint32_t t1 = c1 * deg[v];
            uint32_t t2 = (uint32_t)(P - 1) + T * deg[v];
            acc += (uint64_t)t1 + eta * (uint64_t)t2;
        }
        page_amount[i] = acc;
    }
}

/* std::upper_bound(prefix, prefix + n + 1, x) - 1 - prefix: last index with prefix[j] <= x */
static uint32_t last_le(const uint64_t* prefix, uint32_t n, uint64_t x) {
    uint32_t lo = 0, hi = n + 1; /* first index with prefix > x lies in [lo, hi] */
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (prefix[mid] <= x) lo = mid + 1; else hi = mid;
    }
    return lo - 1;
}

/* judge, core/graph.hpp:586-594: k greedy furthest hops of capacity s reach the end? */
static int judge(uint64_t s, const uint64_t* prefix, uint32_t n, uint32_t k) {
    uint64_t sum = 0;
    for (uint32_t i = 0; i < k; ++i) sum = prefix[last_le(prefix, n, sum + s)];
    return sum == prefix[n];
}

/* optimal_offset, core/graph.hpp:597-626 */
void ora_optimal_offset(const uint64_t* a, uint32_t n, uint32_t k, uint32_t* offset) {
    uint64_t* prefix = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)n + 1));
    prefix[0] = 0;
    for (uint32_t i = 0; i < n; ++i) prefix[i + 1] = prefix[i] + a[i];
    uint64_t lb = prefix[0], ub = prefix[n];
    while (lb + 1 < ub) {
        uint64_t mid = lb + ((ub - lb) >> 1);
        if (judge(mid, prefix, n, k)) ub = mid; else lb = mid;
    }
    offset[0] = 0;
    offset[k] = n;
    uint64_t sum = 0;
    for (uint32_t i = 0; i + 1 < k; ++i) {
        uint32_t j = last_le(prefix, n, sum + ub);
        offset[i + 1] = j;
        sum = prefix[j];
    }
    free(prefix);
}

/* assign_vertices boundaries: core/graph.hpp:718-749 (global) and :774-780 (per partition). */
void ora_cpbt(const uint32_t* deg, uint32_t V, int P, int S, uint64_t eta, int max_iterations,
              int dense, uint32_t* partition_offset, uint32_t* local_offset) {
    uint32_t pages = (V + ORA_PAGESIZE - 1) / ORA_PAGESIZE;
    uint64_t* amount = (uint64_t*)malloc(sizeof(uint64_t) * (pages ? pages : 1));
    uint32_t* page_offset = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)P + 1));
    uint32_t* lpo = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)S + 1));
    ora_page_weights(deg, V, P, eta, max_iterations, dense, amount);
    ora_optimal_offset(amount, pages, (uint32_t)P, page_offset);
    partition_offset[0] = 0;
    partition_offset[P] = V;
    for (int i = 0; i < P - 1; ++i) partition_offset[i + 1] = page_offset[i + 1] * ORA_PAGESIZE;
    if (local_offset) {
        for (int p = 0; p < P; ++p) {
            uint32_t* lo = local_offset + (size_t)p * (S + 1);
            /* pages of partition p: [page_offset[p], page_offset[p+1]) */
            uint32_t pb = page_offset[p], pe = page_offset[p + 1];
            uint32_t cnt = pe >= pb ? pe - pb : 0;
            ora_optimal_offset(amount + pb, cnt, (uint32_t)S, lpo);
            lo[0] = partition_offset[p];
            lo[S] = partition_offset[p + 1];
            for (int i = 0; i < S - 1; ++i) lo[i + 1] = lpo[i + 1] * ORA_PAGESIZE + partition_offset[p];
        }
    }
    free(amount); free(page_offset); free(lpo);
}

/* get_partition_id, core/graph.hpp:404-412 */
int ora_partition_of(const uint32_t* off, int P, uint32_t v) {
    for (int i = 0; i < P; ++i)
        if (v >= off[i] && v < off[i + 1]) return i;
    return -1;
}

/* Stable counting sort of edge ids by (owner partition of okey, skey).  order[] receives the
 * permutation; part_start[P+1] the partition ranges; dense offsets off[P*(V+1)]. */
static void bucket_sort(const uint32_t* okey, const uint32_t* skey, const uint32_t* in_order, uint64_t E,
                        uint32_t V, int P, const uint32_t* poff, uint64_t* part_start, uint64_t* off,
                        uint32_t* order) {
    size_t stride = (size_t)V + 1;
    uint64_t* cnt = (uint64_t*)calloc((size_t)P * stride, sizeof(uint64_t));
    int* owner = (int*)malloc(sizeof(int) * (size_t)V);
    for (uint32_t v = 0; v < V; ++v) owner[v] = ora_partition_of(poff, P, v);
    for (uint64_t i = 0; i < E; ++i) {
        uint64_t e = in_order ? in_order[i] : i;
        cnt[(size_t)owner[okey[e]] * stride + skey[e]]++;
    }
    uint64_t run = 0;
    for (int p = 0; p < P; ++p) {
        part_start[p] = run;
        for (uint32_t v = 0; v < V; ++v) {
            uint64_t c = cnt[(size_t)p * stride + v];
            off[(size_t)p * stride + v] = run;
            cnt[(size_t)p * stride + v] = run;
            run += c;
        }
        off[(size_t)p * stride + V] = run;
    }
    part_start[P] = run;
    for (uint64_t i = 0; i < E; ++i) {
        uint64_t e = in_order ? in_order[i] : i;
        uint64_t pos = cnt[(size_t)owner[okey[e]] * stride + skey[e]]++;
        order[pos] = (uint32_t)e;
    }
    free(cnt); free(owner);
}

void ora_build_csr(const uint32_t* src, const uint32_t* dst, const float* w, uint64_t E, uint32_t V,
                   int P, const uint32_t* poff, uint64_t* part_start, uint64_t* csr_off,
                   uint32_t* csr_dst, float* csr_w, uint64_t* bitmap) {
    uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    bucket_sort(dst, src, NULL, E, V, P, poff, part_start, csr_off, order);
    for (uint64_t i = 0; i < E; ++i) {
        csr_dst[i] = dst[order[i]];
        if (w && csr_w) csr_w[i] = w[order[i]];
    }
    /* outgoing_adj_bitmap, core/graph.hpp:1304-1352: bit u set iff u has an edge in partition p */
    size_t nwords = (size_t)V / 64 + 1, stride = (size_t)V + 1;
    memset(bitmap, 0, sizeof(uint64_t) * nwords * (size_t)P);
    for (int p = 0; p < P; ++p)
        for (uint32_t v = 0; v < V; ++v)
            if (csr_off[p * stride + v + 1] > csr_off[p * stride + v])
                bitmap[p * nwords + v / 64] |= 1ull << (v % 64);
    free(order);
}

uint64_t ora_build_csc(const uint32_t* src, const uint32_t* dst, const float* w, uint64_t E, uint32_t V,
                       int P, const uint32_t* poff, uint64_t* part_start, uint64_t* csc_off,
                       uint32_t* csc_src, float* csc_w, uint64_t* cstart, uint32_t* cvert, uint64_t* cidx,
                       uint64_t ccap) {
    /* first the stable order by src (what prepare_push_mode leaves in edge_list, :1262), then
     * stable by (owner of src, dst) (:1107-1114). */
    uint32_t* by_src = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint64_t* tmp_off = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)V + 1));
    uint64_t tmp_ps[2];
    uint32_t one_part[2] = {0, V};
    bucket_sort(src, src, NULL, E, V, 1, one_part, tmp_ps, tmp_off, by_src);
    bucket_sort(src, dst, by_src, E, V, P, poff, part_start, csc_off, order);
    for (uint64_t i = 0; i < E; ++i) {
        csc_src[i] = src[order[i]];
        if (w && csc_w) csc_w[i] = w[order[i]];
    }
    /* compressed_incoming_adj_index, core/graph.hpp:1144-1188 */
    size_t stride = (size_t)V + 1;
    uint64_t n = 0;
    for (int p = 0; p < P; ++p) {
        cstart[p] = n;
        for (uint32_t v = 0; v < V; ++v) {
            if (csc_off[p * stride + v + 1] > csc_off[p * stride + v]) {
                if (n < ccap) { cvert[n] = v; cidx[n] = csc_off[p * stride + v]; }
                n++;
            }
        }
        if (n < ccap) { cvert[n] = V; cidx[n] = part_start[p + 1]; }
        n++;
    }
    cstart[P] = n;
    free(by_src); free(order); free(tmp_off);
    return n;
}

/* toolkits/pagerank.cpp:26-98 with one partition: dense_signal sums curr[src] over the CSC list
 * (:64-71), dense_slot adds it to next (:72-75), then 1-d+d*next, divided by the out-degree except
 * in the last iteration (:78-98). */
void ora_pagerank(const uint64_t* csc_off, const uint32_t* csc_src, const uint32_t* outdeg,
                  uint32_t V, int iterations, double d, double* out) {
    double* curr = out;
    double* next = (double*)malloc(sizeof(double) * ((size_t)V + 1));
    double* a = curr;
    double* b = next;
    for (uint32_t v = 0; v < V; ++v) {
        a[v] = 1.0;
        if (outdeg[v] > 0) a[v] /= outdeg[v];
    }
    for (int it = 0; it < iterations; ++it) {
        for (uint32_t v = 0; v < V; ++v) {
            double sum = 0;
            for (uint64_t e = csc_off[v]; e < csc_off[v + 1]; ++e) sum += a[csc_src[e]];
            double nx = 0.0 + sum;
            nx = 1 - d + d * nx;
            if (it != iterations - 1 && outdeg[v] > 0) nx /= outdeg[v];
            b[v] = nx;
        }
        double* t = a; a = b; b = t;
    }
    if (a != out) memcpy(out, a, sizeof(double) * V);
    free(next);
}

/* toolkits/bfs.cpp:22-84: push BFS; level[v] = iteration in which v joins active_out, plus one. */
void ora_bfs_levels(const uint64_t* off, const uint32_t* adj, uint32_t V, uint32_t root, uint32_t* level) {
    uint32_t* queue = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)V + 1));
    for (uint32_t v = 0; v < V; ++v) level[v] = ORA_UNREACHED;
    size_t head = 0, tail = 0;
    level[root] = 0;
    queue[tail++] = root;
    while (head < tail) {
        uint32_t u = queue[head++];
        for (uint64_t e = off[u]; e < off[u + 1]; ++e) {
            uint32_t x = adj[e];
            if (level[x] == ORA_UNREACHED) { level[x] = level[u] + 1; queue[tail++] = x; }
        }
    }
    free(queue);
}

uint64_t ora_bfs_check_parents(const uint64_t* off, const uint32_t* adj, uint32_t V, uint32_t root,
                               const uint32_t* level, const uint32_t* parent) {
    /* one pass over the edges marks every vertex whose parent holds an edge to it (O(V + E)) */
    unsigned char* has_edge = (unsigned char*)calloc(V ? V : 1, 1);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t u = 0; u < (int64_t)V; ++u)
        for (uint64_t e = off[u]; e < off[u + 1]; ++e) {
            const uint32_t v = adj[e];
            if (v < V && parent[v] == (uint32_t)u) has_edge[v] = 1;
        }
    uint64_t bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
    for (int64_t i = 0; i < (int64_t)V; ++i) {
        const uint32_t v = (uint32_t)i;
        if (level[v] == ORA_UNREACHED) { bad += parent[v] != V; continue; }
        if (v == root) { bad += parent[v] != root; continue; }
        const uint32_t u = parent[v];
        if (u >= V || level[u] == ORA_UNREACHED || level[u] + 1 != level[v]) { bad++; continue; }
        bad += !has_edge[v];
    }
    free(has_edge);
    return bad;
}

static uint32_t uf_find(uint32_t* par, uint32_t x) {
    while (par[x] != x) { par[x] = par[par[x]]; x = par[x]; }
    return x;
}

/* fixpoint of toolkits/cc.cpp:22-84: every vertex ends with the smallest id of its component */
void ora_cc_labels(const uint32_t* src, const uint32_t* dst, uint64_t E, uint32_t V, uint32_t* label) {
    for (uint32_t v = 0; v < V; ++v) label[v] = v;
    for (uint64_t i = 0; i < E; ++i) {
        uint32_t a = uf_find(label, src[i]), b = uf_find(label, dst[i]);
        if (a < b) label[b] = a; else if (b < a) label[a] = b;
    }
    for (uint32_t v = 0; v < V; ++v) label[v] = uf_find(label, v);
}

/* least fixpoint of toolkits/sssp.cpp:24-84 (relax_dist = msg + w; write_min).  Dijkstra is exact
 * here: fl(x + w) >= x for w >= 0 and fl is monotone, so the extracted minimum is final. */
typedef struct { float d; uint32_t v; } heap_item;
static void heap_push(heap_item* h, size_t* n, heap_item it) {
    size_t i = (*n)++;
    while (i > 0) {
        size_t p = (i - 1) / 2;
        if (h[p].d <= it.d) break;
        h[i] = h[p]; i = p;
    }
    h[i] = it;
}
static heap_item heap_pop(heap_item* h, size_t* n) {
    heap_item top = h[0], last = h[--(*n)];
    size_t i = 0;
    for (;;) {
        size_t l = 2 * i + 1, r = l + 1, m = i;
        float md = last.d;
        if (l < *n && h[l].d < md) { m = l; md = h[l].d; }
        if (r < *n && h[r].d < md) { m = r; }
        if (m == i) break;
        h[i] = h[m]; i = m;
    }
    h[i] = last;
    return top;
}
void ora_sssp(const uint64_t* off, const uint32_t* adj, const float* w, uint32_t V, uint32_t root, float* dist) {
    for (uint32_t v = 0; v < V; ++v) dist[v] = 1e9f;
    uint64_t E = off[V];
    heap_item* h = (heap_item*)malloc(sizeof(heap_item) * (E + 2));
    size_t n = 0;
    dist[root] = 0.f;
    heap_item it0 = {0.f, root};
    heap_push(h, &n, it0);
    while (n) {
        heap_item it = heap_pop(h, &n);
        if (it.d > dist[it.v]) continue;
        uint32_t u = it.v;
        for (uint64_t e = off[u]; e < off[u + 1]; ++e) {
            float nd = dist[u] + w[e];
            if (nd < dist[adj[e]]) {
                dist[adj[e]] = nd;
                heap_item ni = {nd, adj[e]};
                heap_push(h, &n, ni);
            }
        }
    }
    free(h);
}

void ora_bc(const uint64_t* off, const uint32_t* adj, uint32_t V, uint32_t root, double* sigma, double* delta,
            uint32_t* level) {
    uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * (V ? V : 1));
    for (uint32_t v = 0; v < V; ++v) {
        sigma[v] = 0.0;
        delta[v] = 0.0;
        level[v] = ORA_UNREACHED;
    }
    uint32_t head = 0, tail = 0;
    sigma[root] = 1.0;
    level[root] = 0;
    order[tail++] = root;
    while (head < tail) {
        const uint32_t v = order[head++];
        for (uint64_t e = off[v]; e < off[v + 1]; ++e) {
            const uint32_t w = adj[e];
            if (level[w] == ORA_UNREACHED) {
                level[w] = level[v] + 1;
                order[tail++] = w;
            }
            if (level[w] == level[v] + 1) sigma[w] += sigma[v];
        }
    }
    for (uint32_t i = tail; i-- > 0;) {
        const uint32_t w = order[i];
        for (uint64_t e = off[w]; e < off[w + 1]; ++e) {
            const uint32_t x = adj[e];
            if (level[x] == level[w] + 1) delta[w] += sigma[w] / sigma[x] * (1.0 + delta[x]);
        }
    }
    free(order);
}

void ora_adjacency_hash(const uint32_t* src, const uint32_t* dst, const float* w, uint64_t E, uint32_t V,
                        uint64_t* hout, uint64_t* hin) {
    memset(hout, 0, sizeof(uint64_t) * V);
    memset(hin, 0, sizeof(uint64_t) * V);
    for (uint64_t i = 0; i < E; ++i) {
        uint64_t wb = 0;
        if (w) { uint32_t b; memcpy(&b, &w[i], 4); wb = (uint64_t)b << 32; }
        hout[src[i]] += eg_mix64(dst[i] | wb);
        hin[dst[i]] += eg_mix64(src[i] | wb);
    }
}

void ora_list_hash(const uint64_t* off, const uint32_t* adj, const float* w, uint64_t n, uint64_t* h) {
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
        uint64_t acc = 0;
        for (uint64_t e = off[v]; e < off[v + 1]; ++e) {
            uint64_t wb = 0;
            if (w) { uint32_t b; memcpy(&b, &w[e], 4); wb = (uint64_t)b << 32; }
            acc += eg_mix64(adj[e] | wb);
        }
        h[v] = acc;
    }
}
