// endgraph_gb300_engine.cuh — Gemini's process_edges / process_vertices (core/graph.hpp:1376-1817
// of the reference) for operators written as device functors, on a graph that libendgraph_gb300
// has loaded and built (eg_load_directed / eg_load_undirected_from_directed).  Header-only host
// and device code: include it from a .cu file compiled for sm_103a and link the library.
//
// The reference passes four host lambdas (sparse_signal, sparse_slot, dense_signal, dense_slot)
// that the engine calls per vertex and per adjacency list.  Here the same four roles are device
// member functions of one operator type, split per edge so that the engine can balance hubs and
// leaves (rank-balanced push over the frontier's out-edges; chunked pull over the CSC):
//
//   struct Op {
//     using Msg = ...;  // sparse message (any trivially copyable type)
//     using Acc = ...;  // dense reduction (4 or 8 bytes, trivially copyable)
//     using R   = ...;  // value summed over slots: int, unsigned, unsigned long long, float or double
//     // sparse (push): for every vertex of the active subset; true = emit(v, msg)
//     __device__ bool sparse_signal(uint32_t v, Msg& msg) const;
//     // for every out-edge (v, dst, w) of an emitting vertex (w = 0 on unweighted graphs)
//     __device__ R sparse_slot(uint32_t v, const Msg& msg, uint32_t dst, float w) const;
//     // dense (pull): destinations to reduce into (the reference's dense_signal returns early for
//     // the others)
//     __device__ bool dense_active(uint32_t dst) const;
//     __device__ Acc dense_identity() const;
//     // contribution of in-edge (src, dst, w); the identity contributes nothing
//     __device__ Acc dense_signal(uint32_t src, float w) const;
//     __device__ Acc dense_combine(Acc a, Acc b) const;
//     // once per active destination with in-edges, with the reduction over all of its in-edges
//     // (the identity when none contributed)
//     __device__ R dense_slot(uint32_t dst, Acc acc) const;
//   };
//
// With several CPBT partitions the engine runs Gemini's master/mirror message path
// (core/graph.hpp:1445-1470, :1505-1802) over per-partition message buffers in device memory --
// exactly what a multi-GPU build would exchange between ranks:
//   sparse  every active master signals into the buffer of the partition that owns it
//           ({vertex, msg} pairs, emit :1460); every partition then relaxes the messages of all
//           buffers along its own CSR lists (the mirrors' slots, :1590-1655)
//   dense   every partition reduces its in-edges (sources it owns) per destination and sends the
//           partial to the destination's master partition as one {vertex, partial} message; each
//           master buffer is then handed to dense_slot message by message (:1684-1801)
// so dense_slot may see several partials of one destination, as in the reference; the slots of
// the four toolkits combine them (write_add, cas, write_min).  With one partition, or with the
// message path switched off, dense_slot sees the complete reduction of a destination once.
// dense_selective (:1666-1682) is the subset the dense signals read; the reference sends each
// rank's owned slice to every other rank first.  Here every partition reads the same device words,
// so nothing moves; the slice volume is counted in message_stats() as what that exchange carries.
// Slots run concurrently and must use atomics for shared state, as the reference's slots do
// (core/atomic.hpp); a destination's contributions combine in any order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "endgraph_gb300.h"
#include "endgraph_gb300_kernels.cuh"

namespace eg {
namespace engine {

class Error : public std::runtime_error {
   public:
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Error(EG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
inline void check_eg(int st, const char* what) {
    if (st != EG_OK) throw Error(st, std::string(what) + ": " + eg_last_error());
}

// VertexSubset (core/bitmap.hpp:23-68) in device memory: bit v of words[v / 64]
struct Subset {
    unsigned long long* words = nullptr;
    uint32_t V = 0;
    __device__ __forceinline__ bool get_bit(uint32_t v) const { return (__ldcg(words + (v >> 6)) >> (v & 63)) & 1ull; }
    __device__ __forceinline__ void set_bit(uint32_t v) const { atomicOr(words + (v >> 6), 1ull << (v & 63)); }
    size_t nwords() const { return (size_t)V / 64 + 1; }
};

enum class Mode { Auto, Sparse, Dense };

namespace detail {

template <class T>
__device__ __forceinline__ auto to_bits(T v) {
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "dense accumulators are 4 or 8 bytes");
    using U = std::conditional_t<sizeof(T) == 4, unsigned int, unsigned long long>;
    U u;
    memcpy(&u, &v, sizeof(T));
    return u;
}
template <class T, class U>
__device__ __forceinline__ T from_bits(U u) {
    T v;
    memcpy(&v, &u, sizeof(T));
    return v;
}
// *p = comb(*p, v) atomically (shared or global memory)
template <class T, class C>
__device__ __forceinline__ void atomic_combine(T* p, T v, const C& comb) {
    using U = decltype(to_bits(v));
    U* a = reinterpret_cast<U*>(p);
    U old = *reinterpret_cast<volatile U*>(a);
    while (true) {
        const U nw = to_bits(comb(from_bits<T>(old), v));
        if (nw == old) return;
        const U seen = atomicCAS(a, old, nw);
        if (seen == old) return;
        old = seen;
    }
}
template <class R>
__device__ __forceinline__ void warp_add_out(R r, R* out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if ((threadIdx.x & 31) == 0 && r != R(0)) atomicAdd(out, r);
}

template <class Op>
struct PushAdapter {
    using Msg = typename Op::Msg;
    using Value = typename Op::R;
    Op op;
    const Msg* msg;
    const float* w;
    Value* out;
    __device__ Msg payload(uint32_t u) const { return msg[u]; }
    __device__ bool relax(uint32_t u, const Msg& m, uint32_t dst, uint64_t pos, Value& acc) const {
        acc += op.sparse_slot(u, m, dst, w ? w[pos] : 0.f);
        return false;
    }
    __device__ void reduce_out(Value v) const {
        if (v != Value(0)) atomicAdd(out, v);
    }
};

template <class Op>
struct PullAdapter {
    using Acc = typename Op::Acc;
    using R = typename Op::R;
    static constexpr bool kFilter = true;
    Op op;
    const float* w;
    Acc* partial;  // [V] combined partial reductions of destinations split across chunks
    R* out;
    int single;    // one partition: an item wholly inside a chunk is the whole destination
    __device__ bool stopped() const { return false; }
    __device__ bool item_active(uint32_t v) const { return op.dense_active(v); }
    __device__ Acc identity() const { return op.dense_identity(); }
    __device__ Acc gather(uint32_t u, uint64_t pos) const { return op.dense_signal(u, w ? w[pos] : 0.f); }
    __device__ Acc combine(Acc a, Acc b) const { return op.dense_combine(a, b); }
    __device__ void smem_add(Acc* slot, Acc v) const {
        if (to_bits(v) != to_bits(identity()))
            atomic_combine(slot, v, [this](Acc x, Acc y) { return op.dense_combine(x, y); });
    }
    __device__ void finish(bool ok, uint32_t v, Acc a, bool whole) const {
        R r = R(0);
        if (ok && op.dense_active(v)) {
            if (whole && single) {
                r = op.dense_slot(v, a);
            } else if (to_bits(a) != to_bits(identity())) {
                atomic_combine(partial + v, a, [this](Acc x, Acc y) { return op.dense_combine(x, y); });
            }
        }
        warp_add_out(r, out);
    }
};

// owner partition of v: last i with part_off[i] <= v (part_off: P+1 monotone offsets, v < part_off[P])
__device__ __forceinline__ int owner_of(const uint32_t* __restrict__ part_off, int P, uint32_t v) {
    int lo = 0, hi = P;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (part_off[mid] <= v) lo = mid; else hi = mid;
    }
    return lo;
}

// message path, sparse signal: active masters emit into their own partition's buffer, which
// starts at part_off[p] (a partition emits at most one message per vertex it owns)
template <class Op>
__global__ void k_signal_msgs(Op op, const uint32_t* __restrict__ q, const uint32_t* nq,
                              const uint32_t* __restrict__ part_off, int P, uint32_t* __restrict__ mvert,
                              typename Op::Msg* __restrict__ mdata, uint32_t* __restrict__ mcount) {
    const uint32_t n = __ldcg(nq);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = q[i];
        typename Op::Msg m;
        if (op.sparse_signal(v, m)) {
            const int p = owner_of(part_off, P, v);
            const uint32_t at = part_off[p] + atomicAdd(mcount + p, 1u);
            mvert[at] = v;
            mdata[at] = m;
        }
    }
}

// message path, sparse receive: the buffers of all partitions, concatenated in partition order,
// become the emitter queue of the slot pass and their payloads its per-vertex messages
template <class Msg>
__global__ void k_recv_msgs(const uint32_t* __restrict__ mvert, const Msg* __restrict__ mdata,
                            const uint32_t* __restrict__ part_off, const uint32_t* __restrict__ mcount, int P,
                            Msg* __restrict__ payload, uint32_t* __restrict__ q) {
    uint32_t base = 0;
    for (int p = 0; p < P; ++p) {
        const uint32_t n = mcount[p];
        for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
            const uint32_t at = part_off[p] + j;
            const uint32_t v = mvert[at];
            payload[v] = mdata[at];
            q[base + j] = v;
        }
        base += n;
    }
}

// message path, dense slots: every master partition's buffer, message by message
template <class Op>
__global__ void k_slot_msgs(Op op, const uint32_t* __restrict__ dvert, const typename Op::Acc* __restrict__ ddata,
                            const uint64_t* __restrict__ dbase, const uint32_t* __restrict__ dcount, int P,
                            typename Op::R* out) {
    using R = typename Op::R;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (int i = 0; i < P; ++i) {
        const uint64_t n = dcount[i], b = dbase[i];
        for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
            const uint64_t j = base + threadIdx.x;
            R r = R(0);
            if (j < n) r = op.dense_slot(dvert[b + j], ddata[b + j]);
            warp_add_out(r, out);
        }
    }
}

// message buffers per master partition of the dense path: entries with the destination's owner
template <class Op>
struct PullMsgAdapter {
    using Acc = typename Op::Acc;
    static constexpr bool kFilter = true;
    Op op;
    const float* w;
    const uint32_t* part_off;
    int P;
    uint32_t* dvert;
    Acc* ddata;
    const uint64_t* dbase;  // [P+1] buffer starts; dbase[i+1] - dbase[i] = capacity of buffer i
    uint32_t* dcount;
    int* overflow;
    __device__ bool stopped() const { return false; }
    __device__ bool item_active(uint32_t v) const { return op.dense_active(v); }
    __device__ Acc identity() const { return op.dense_identity(); }
    __device__ Acc gather(uint32_t u, uint64_t pos) const { return op.dense_signal(u, w ? w[pos] : 0.f); }
    __device__ Acc combine(Acc a, Acc b) const { return op.dense_combine(a, b); }
    __device__ void smem_add(Acc* slot, Acc v) const {
        if (to_bits(v) != to_bits(identity()))
            atomic_combine(slot, v, [this](Acc x, Acc y) { return op.dense_combine(x, y); });
    }
    // one message per reduced piece of a (partition, destination) list; a list that crosses chunk
    // boundaries sends one partial per chunk
    __device__ void finish(bool ok, uint32_t v, Acc a, bool) const {
        if (!ok || !op.dense_active(v) || to_bits(a) == to_bits(identity())) return;
        const int i = owner_of(part_off, P, v);
        const uint64_t at = dbase[i] + atomicAdd(dcount + i, 1u);
        if (at < dbase[i + 1]) {
            dvert[at] = v;
            ddata[at] = a;
        } else {
            atomicExch(overflow, 1);
        }
    }
};

template <class Op>
__global__ void k_sparse_signal(Op op, const uint32_t* __restrict__ q, const uint32_t* nq, typename Op::Msg* msg,
                                uint32_t* q_out, uint32_t* n_out) {
    __shared__ uint32_t s_cnt[2 * (1024 / 32 + 1)];
    const uint32_t n = __ldcg(nq);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint64_t i = base + threadIdx.x;
        bool emit = false;
        uint32_t v = 0;
        if (i < n) {
            v = q[i];
            typename Op::Msg m;
            emit = op.sparse_signal(v, m);
            if (emit) msg[v] = m;
        }
        append_block(emit, v, q_out, n_out, s_cnt, 0);  // the loop is uniform across the CTA
    }
}

template <class Op>
__global__ void k_fill_acc(typename Op::Acc* p, uint64_t n, Op op) {
    const typename Op::Acc id = op.dense_identity();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = id;
}

// destinations whose reduction was combined in `partial`: the split list (one partition) or every
// vertex with in-edges (several partitions)
template <class Op>
__global__ void k_dense_finish(Op op, const uint32_t* __restrict__ split, const uint32_t* __restrict__ cvert,
                               uint64_t nsplit, const uint32_t* __restrict__ indeg, uint32_t V,
                               typename Op::Acc* partial, typename Op::R* out) {
    using R = typename Op::R;
    const uint64_t n = split ? nsplit : V;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint64_t i = base + threadIdx.x;
        R r = R(0);
        if (i < n) {
            const uint32_t v = split ? cvert[split[i]] : (uint32_t)i;
            if (v < V && (split || indeg[v] > 0) && op.dense_active(v)) {
                const typename Op::Acc a = partial[v];
                partial[v] = op.dense_identity();
                r = op.dense_slot(v, a);
            }
        }
        warp_add_out(r, out);
    }
}

template <class R, class F>
__global__ void k_vertices(F f, const unsigned long long* __restrict__ words, uint64_t nwords, uint32_t V, R* out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < nwords; base += stride) {
        const uint64_t w = base + threadIdx.x;
        R r = R(0);
        if (w < nwords) {
            unsigned long long word = words[w];
            while (word) {
                const uint32_t v = (uint32_t)(w * 64 + (uint64_t)(__ffsll((long long)word) - 1));
                word &= word - 1;
                if (v < V) r += f(v);
            }
        }
        warp_add_out(r, out);
    }
}

// compressed items per owner partition of their destination (dense message buffer capacities)
static __global__ void k_items_per_owner(const uint32_t* __restrict__ cvert, uint64_t nitems, uint32_t V,
                                         const uint32_t* __restrict__ part_off, int P, unsigned long long* cnt) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nitems; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = cvert[i];
        if (v < V) atomicAdd(cnt + owner_of(part_off, P, v), 1ull);
    }
}

static __global__ void k_fill_words(unsigned long long* words, uint64_t nwords, uint32_t V) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords; w += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t lo = w * 64;
        unsigned long long x = 0;
        if (lo + 64 <= V) x = ~0ull;
        else if (lo < V) x = (1ull << (V - lo)) - 1ull;
        words[w] = x;
    }
}

// ordered compaction of the vertices with out-edges into a compressed index over the CSR (the
// pull side of the transposed graph), closed by a {V, E} sentinel
struct LoadHasOut {
    const uint32_t* deg;
    uint32_t V;
    __device__ uint32_t operator()(uint64_t i) const { return i >= V ? 1u : (deg[i] > 0 ? 1u : 0u); }
};
struct EpiRowIndex {
    const uint64_t* off;
    uint32_t V;
    uint64_t E;
    uint32_t* cvert;
    uint64_t* cidx;
    __device__ void operator()(uint64_t i, uint64_t excl, uint32_t flag) const {
        if (!flag) return;
        cvert[excl] = i >= V ? V : (uint32_t)i;
        cidx[excl] = i >= V ? E : off[i];
    }
};

}  // namespace detail

// One engine per built graph.  All work is ordered on the graph handle's stream; the results of
// process_edges / process_vertices are returned to the host (one synchronisation per call).
class Engine {
   public:
    explicit Engine(eg_graph* g) : g_(g) {
        eg_info info;
        check_eg(eg_get_info(g, &info), "eg_get_info");
        if (!info.built_csr || !info.built_csc) throw Error(EG_ERR_STATE, "Engine: build CSR and CSC first");
        V_ = info.V;
        E_ = info.E;
        P_ = (int)info.partitions;
        check_eg(eg_get_csr(g, &csr_), "eg_get_csr");
        check_eg(eg_get_csc(g, &csc_), "eg_get_csc");
        stream_ = (cudaStream_t)eg_stream(g);
        int dev = 0;
        check(cudaGetDevice(&dev), "cudaGetDevice");
        check(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
        outdeg_ = alloc<uint32_t>(V_);
        indeg_ = alloc<uint32_t>(V_);
        check_eg(eg_get_degrees(g, outdeg_, indeg_, EG_DEVICE), "eg_get_degrees");
        counters_ = alloc<unsigned long long>(8);
        q0_ = alloc<uint32_t>((size_t)V_ + 1);
        q1_ = alloc<uint32_t>((size_t)V_ + 1);
        ipref_ = alloc<uint64_t>((size_t)V_ * P_ + 2);
        push_chunk_ = alloc<uint32_t>(E_ / kPushChunk + 4);
        scan_desc_ = alloc<uint64_t>(((size_t)V_ * P_ + kScanTile) / kScanTile + 2);
        // as built: push along the CSR, pull over the compressed CSC
        Side& f = side_[0];
        f.push_off = csr_.off;
        f.push_adj = csr_.adj;
        f.push_w = csr_.w;
        f.push_deg = outdeg_;
        f.pull_adj = csc_.adj;
        f.pull_w = csc_.w;
        f.pull_cvert = csc_.cvert;
        f.pull_cidx = csc_.cidx;
        f.pull_deg = indeg_;
        f.nitems = info.ncompressed - 1;
        setup_pull_chunks(f);
        cur_ = &side_[0];
        // CPBT partition offsets (the masters of each partition), host and device copies
        h_part_off_.assign((size_t)P_ + 1, 0);
        check_eg(eg_get_partition(g, h_part_off_.data(), nullptr), "eg_get_partition");
        for (int i = 1; i <= P_; ++i) h_part_off_[i] = std::max(std::min(h_part_off_[i], V_), h_part_off_[i - 1]);
        part_off_ = alloc<uint32_t>((size_t)P_ + 1);
        check(cudaMemcpyAsync(part_off_, h_part_off_.data(), 4 * ((size_t)P_ + 1), cudaMemcpyHostToDevice, stream_),
              "part_off");
        check(cudaStreamSynchronize(stream_), "part_off");
        msg_path_ = P_ > 1;
    }
    ~Engine() {
        for (void* p : {(void*)outdeg_, (void*)indeg_, (void*)counters_, (void*)q0_, (void*)q1_, (void*)ipref_,
                        (void*)push_chunk_, (void*)scan_desc_, msg_, partial_, (void*)row_cvert_, (void*)row_cidx_,
                        (void*)part_off_, (void*)mvert_, mdata_, (void*)mcount_, (void*)dvert_, ddata_, (void*)dbase_,
                        (void*)dcount_})
            if (p) cudaFree(p);
        for (Side& sd : side_)
            for (void* p : {(void*)sd.chunk, (void*)sd.split})
                if (p) cudaFree(p);
    }
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    uint32_t vertices() const { return V_; }
    uint64_t edges() const { return E_; }
    cudaStream_t stream() const { return stream_; }
    const uint32_t* out_degree() const { return outdeg_; }  // device
    const uint32_t* in_degree() const { return indeg_; }    // device
    bool last_was_dense() const { return last_dense_; }

    // process_edges on the transposed graph: push along in-edges (the CSC lists) and pull over
    // out-edges (the CSR lists, indexed on first use) -- the reverse sweeps of a backward pass
    // (the reference's transpose(), core/graph.hpp:649-657, swaps the same two structures).
    // Degrees, the switch's active-edge count and process_edges' roles follow the orientation.
    // One partition only.
    void set_transposed(bool t) {
        if (t && P_ != 1) throw Error(EG_ERR_UNSUPPORTED, "set_transposed: one partition only");
        if (t && !side_[1].ready) setup_transposed();
        cur_ = &side_[t ? 1 : 0];
    }
    bool transposed() const { return cur_ == &side_[1]; }
    uint64_t last_active_edges() const { return last_active_edges_; }

    // The master/mirror message path over per-partition buffers (on by default with several
    // partitions; off: the shared-memory engine, which needs no buffers and gives dense_slot the
    // complete reduction of a destination).  As built only: the transposed graph has one partition.
    void set_message_path(bool on) { msg_path_ = on && P_ > 1; }
    bool message_path() const { return msg_path_; }
    // what the last process_edges put in the partitions' buffers: messages per partition (sparse:
    // by the master that emitted them; dense: by the master they are addressed to), and the bytes a
    // rank-per-partition run would send: each sparse buffer to P-1 ranks, each dense message once
    // (an upper bound: a partition's partials for its own masters stay local), and each rank's slice
    // of dense_selective to P-1 ranks
    struct MessageStats {
        uint64_t messages = 0;
        uint64_t bytes = 0;
        uint64_t selective_bytes = 0;
        std::vector<uint64_t> per_partition;
    };
    const MessageStats& message_stats() const { return stats_; }
    const std::vector<uint32_t>& partition_offsets() const { return h_part_off_; }

    // vertex arrays and subsets in device memory (alloc_vertex_array / alloc_vertex_subset)
    template <class T>
    T* alloc_vertex_array() {
        return alloc<T>(V_);
    }
    template <class T>
    void fill_vertex_array(T* a, T value) {
        std::vector<T> h((size_t)V_, value);
        check(cudaMemcpyAsync(a, h.data(), sizeof(T) * (size_t)V_, cudaMemcpyHostToDevice, stream_), "fill");
        check(cudaStreamSynchronize(stream_), "fill");
    }
    void free(void* p) { cudaFree(p); }
    Subset alloc_subset() {
        Subset s;
        s.V = V_;
        s.words = alloc<unsigned long long>(s.nwords());
        clear(s);
        return s;
    }
    void free_subset(Subset& s) {
        cudaFree(s.words);
        s.words = nullptr;
    }
    void clear(const Subset& s) { check(cudaMemsetAsync(s.words, 0, 8 * s.nwords(), stream_), "clear"); }
    void fill(const Subset& s) {
        detail::k_fill_words<<<grid(s.nwords()), 256, 0, stream_>>>(s.words, s.nwords(), V_);
        check(cudaGetLastError(), "k_fill_words");
    }
    void set_bit(const Subset& s, uint32_t v) {  // host-side, stream-ordered
        if (v >= V_) throw Error(EG_ERR_INVALID, "set_bit: vertex out of range");
        unsigned long long word = 0;
        check(cudaMemcpyAsync(&word, s.words + (v >> 6), 8, cudaMemcpyDeviceToHost, stream_), "set_bit");
        check(cudaStreamSynchronize(stream_), "set_bit");
        word |= 1ull << (v & 63);
        check(cudaMemcpyAsync(s.words + (v >> 6), &word, 8, cudaMemcpyHostToDevice, stream_), "set_bit");
        check(cudaStreamSynchronize(stream_), "set_bit");
    }

    // sum of f(v) over the vertices of `active` (core/graph.hpp:1377-1441); f is a device functor
    template <class R, class F>
    R process_vertices(const F& f, const Subset& active) {
        R* out = reinterpret_cast<R*>(counters_ + 6);
        check(cudaMemsetAsync(out, 0, sizeof(R), stream_), "cudaMemsetAsync");
        detail::k_vertices<R, F><<<grid(active.nwords()), 256, 0, stream_>>>(f, active.words, active.nwords(), V_, out);
        check(cudaGetLastError(), "k_vertices");
        R h{};
        check(cudaMemcpyAsync(&h, out, sizeof(R), cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        return h;
    }

    // core/graph.hpp:1473-1817.  Auto takes the sparse (push) path iff the active vertices' out-edges
    // are fewer than E / dense_divisor (the reference's E / 20, :1484-1491); the dense path does not
    // read `active` (an operator's dense_signal consults it, as the reference's dense_signal does).
    // dense_selective: the subset the operator's dense signals read (the reference's
    // process_edges argument); see the header comment for what happens to it.
    template <class Op>
    typename Op::R process_edges(const Op& op, const Subset& active, Mode mode = Mode::Auto, int dense_divisor = 20,
                                 const Subset* dense_selective = nullptr) {
        using R = typename Op::R;
        static_assert(std::is_trivially_copyable<Op>::value, "operators are passed to kernels by value");
        if (active.V != V_ || (dense_selective && dense_selective->V != V_))
            throw Error(EG_ERR_INVALID, "process_edges: subsets must hold the graph's vertices");
        stats_ = MessageStats();
        stats_.per_partition.assign((size_t)P_, 0);
        R* out = reinterpret_cast<R*>(counters_ + 6);
        check(cudaMemsetAsync(out, 0, sizeof(R), stream_), "cudaMemsetAsync");
        uint32_t* d_n = reinterpret_cast<uint32_t*>(counters_ + 2);
        unsigned long long* d_act = counters_ + 3;
        bool dense = mode == Mode::Dense;
        uint32_t n_active = 0;
        if (mode != Mode::Dense) {
            check(cudaMemsetAsync(counters_ + 2, 0, 16, stream_), "cudaMemsetAsync");
            k_bm_compact<<<grid(active.nwords()), 256, 0, stream_>>>(active.words, active.nwords(), q0_, d_n, d_act,
                                                                     cur_->push_deg);
            check(cudaGetLastError(), "k_bm_compact");
            struct {
                uint32_t n, pad;
                unsigned long long act;
            } h;
            check(cudaMemcpyAsync(&h, counters_ + 2, 16, cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
            check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
            n_active = h.n;
            last_active_edges_ = h.act;
            dense = mode == Mode::Auto && h.act >= E_ / (uint64_t)std::max(dense_divisor, 1);
        }
        last_dense_ = dense;
        if (dense && dense_selective && msg_path_) {
            for (int i = 0; i < P_; ++i)
                stats_.selective_bytes +=
                    8ull * ((h_part_off_[i + 1] - h_part_off_[i]) / 64) * (uint64_t)(P_ - 1);
        }
        if (dense) {
            if (msg_path_) run_dense_msgs(op, out);
            else run_dense(op, out);
        } else if (n_active) {
            if (msg_path_) run_sparse_msgs(op, n_active, out);
            else run_sparse(op, n_active, out);
        }
        R h{};
        check(cudaMemcpyAsync(&h, out, sizeof(R), cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        return h;
    }

   private:
    struct Side {
        const uint64_t* push_off = nullptr;  // [P*(V+1)] list offsets of the push direction
        const uint32_t* push_adj = nullptr;
        const float* push_w = nullptr;
        const uint32_t* push_deg = nullptr;  // list lengths (active-edge count of the switch)
        const uint32_t* pull_adj = nullptr;
        const float* pull_w = nullptr;
        const uint32_t* pull_cvert = nullptr;  // compressed index of the pull direction
        const uint64_t* pull_cidx = nullptr;
        const uint32_t* pull_deg = nullptr;
        uint64_t nitems = 0, nchunks = 0;
        uint32_t* chunk = nullptr;  // first compressed entry per 4096-edge chunk
        uint32_t* split = nullptr;  // entries whose list crosses a chunk boundary
        unsigned long long nsplit = 0;
        bool ready = false;
    };

    template <class T>
    T* alloc(size_t n) {
        void* p = nullptr;
        check(cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)), "cudaMalloc");
        return static_cast<T*>(p);
    }
    unsigned grid(uint64_t n, unsigned block = 256) const {
        uint64_t b = (n + block - 1) / block;
        b = std::max<uint64_t>(b, 1);
        return (unsigned)std::min<uint64_t>(b, (uint64_t)num_sms_ * 16u);
    }

    template <class Op>
    void run_sparse(const Op& op, uint32_t n_active, typename Op::R* out) {
        using Msg = typename Op::Msg;
        ensure_msg_arrays<Msg>();
        Msg* msg = static_cast<Msg*>(msg_);
        uint32_t* d_n = reinterpret_cast<uint32_t*>(counters_ + 2);
        uint32_t* d_emit = reinterpret_cast<uint32_t*>(counters_ + 4);
        check(cudaMemsetAsync(d_emit, 0, 4, stream_), "cudaMemsetAsync");
        detail::k_sparse_signal<Op><<<grid(n_active), 256, 0, stream_>>>(op, q0_, d_n, msg, q1_, d_emit);
        check(cudaGetLastError(), "k_sparse_signal");
        uint32_t n_emit = 0;
        check(cudaMemcpyAsync(&n_emit, d_emit, 4, cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        if (n_emit) push_emitters(op, msg, n_emit, out);
    }

    // master/mirror sparse step: masters signal into their partition's buffer; every partition
    // relaxes all buffers along its own lists (the buffers, concatenated, are the emitter queue)
    template <class Op>
    void run_sparse_msgs(const Op& op, uint32_t n_active, typename Op::R* out) {
        using Msg = typename Op::Msg;
        ensure_msg_arrays<Msg>();
        if (!mvert_) mvert_ = alloc<uint32_t>(V_);
        if (mdata_bytes_ < sizeof(Msg) * (size_t)V_) {
            if (mdata_) cudaFree(mdata_);
            mdata_ = nullptr;
            check(cudaMalloc(&mdata_, sizeof(Msg) * (size_t)V_), "cudaMalloc");
            mdata_bytes_ = sizeof(Msg) * (size_t)V_;
        }
        if (!mcount_) mcount_ = alloc<uint32_t>((size_t)P_);
        check(cudaMemsetAsync(mcount_, 0, 4 * (size_t)P_, stream_), "cudaMemsetAsync");
        uint32_t* d_n = reinterpret_cast<uint32_t*>(counters_ + 2);
        detail::k_signal_msgs<Op><<<grid(n_active), 256, 0, stream_>>>(op, q0_, d_n, part_off_, P_, mvert_,
                                                                      static_cast<Msg*>(mdata_), mcount_);
        check(cudaGetLastError(), "k_signal_msgs");
        std::vector<uint32_t> cnt((size_t)P_);
        check(cudaMemcpyAsync(cnt.data(), mcount_, 4 * (size_t)P_, cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        uint64_t n_emit = 0;
        for (int p = 0; p < P_; ++p) {
            n_emit += cnt[p];
            stats_.per_partition[p] = cnt[p];
        }
        stats_.messages = n_emit;
        stats_.bytes = n_emit * (sizeof(uint32_t) + sizeof(Msg)) * (uint64_t)(P_ - 1);
        if (!n_emit) return;
        Msg* payload = static_cast<Msg*>(msg_);
        detail::k_recv_msgs<Msg><<<grid(n_emit), 256, 0, stream_>>>(mvert_, static_cast<const Msg*>(mdata_), part_off_,
                                                                   mcount_, P_, payload, q1_);
        check(cudaGetLastError(), "k_recv_msgs");
        push_emitters(op, payload, (uint32_t)n_emit, out);
    }

    template <class Msg>
    void ensure_msg_arrays() {
        if (msg_bytes_ < sizeof(Msg) * (size_t)V_) {
            if (msg_) cudaFree(msg_);
            msg_ = nullptr;
            check(cudaMalloc(&msg_, sizeof(Msg) * (size_t)V_), "cudaMalloc");
            msg_bytes_ = sizeof(Msg) * (size_t)V_;
        }
    }

    // relax the out-edges (every partition's list) of the n_emit emitters queued in q1_, whose
    // messages are msg[v]
    template <class Op>
    void push_emitters(const Op& op, const typename Op::Msg* msg, uint32_t n_emit, typename Op::R* out) {
        // ranks of the emitters' out-edges (every partition's list of every emitter)
        const uint64_t nitems = (uint64_t)n_emit * P_;
        const uint64_t tiles = std::max<uint64_t>((nitems + kScanTile - 1) / kScanTile, 1);
        check(cudaMemsetAsync(scan_desc_, 0, 8 * tiles, stream_), "cudaMemsetAsync");
        check(cudaMemsetAsync(counters_ + 5, 0, 8, stream_), "cudaMemsetAsync");  // ticket + error flag
        uint32_t* ticket = reinterpret_cast<uint32_t*>(counters_ + 5);
        int* err = reinterpret_cast<int*>(ticket + 1);
        const Side& sd = *cur_;
        LoadItemLen ld{q1_, P_, (uint64_t)V_ + 1, sd.push_off};
        EpiItemRank ep{ipref_, push_chunk_};
        k_scan<<<(unsigned)tiles, kScanThreads, 0, stream_>>>(ld, ep, nitems, scan_desc_, ticket, err, ipref_ + nitems,
                                                             kLookbackSpinCap);
        check(cudaGetLastError(), "k_scan");
        PushArgs a;
        a.q = q1_;
        a.nitems = nitems;
        a.P = P_;
        a.stride = (uint64_t)V_ + 1;
        a.off = sd.push_off;
        a.adj = sd.push_adj;
        a.w = sd.push_w;
        a.ipref = ipref_;
        a.chunk_item = push_chunk_;
        a.q_out = nullptr;
        a.n_out = nullptr;
        a.act_edges = nullptr;
        a.deg = nullptr;
        detail::PushAdapter<Op> pa{op, msg, sd.push_w, out};
        k_push<detail::PushAdapter<Op>><<<(unsigned)num_sms_ * 8u, kPushThreads, 0, stream_>>>(pa, a);
        check(cudaGetLastError(), "k_push");
        int h_err = 0;
        check(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        if (h_err) throw Error(EG_ERR_TIMEOUT, "process_edges: a bounded device wait gave up");
    }

    template <class Op>
    void run_dense(const Op& op, typename Op::R* out) {
        using Acc = typename Op::Acc;
        const Side& sd = *cur_;
        if (sd.nchunks == 0) return;
        // partial reductions start at the operator's identity
        const typename Op::Acc id = host_identity(op);
        unsigned long long id_bits = 0;
        memcpy(&id_bits, &id, sizeof(Acc));
        if (partial_bytes_ < sizeof(Acc) * (size_t)V_ || partial_size_ != sizeof(Acc) || partial_id_ != id_bits) {
            if (partial_bytes_ < sizeof(Acc) * (size_t)V_) {
                if (partial_) cudaFree(partial_);
                partial_ = nullptr;
                check(cudaMalloc(&partial_, sizeof(Acc) * (size_t)V_), "cudaMalloc");
                partial_bytes_ = sizeof(Acc) * (size_t)V_;
            }
            detail::k_fill_acc<Op><<<grid(V_), 256, 0, stream_>>>(static_cast<Acc*>(partial_), V_, op);
            check(cudaGetLastError(), "k_fill_acc");
            partial_size_ = sizeof(Acc);
            partial_id_ = id_bits;
        }
        detail::PullAdapter<Op> pa{op, sd.pull_w, static_cast<Acc*>(partial_), out, P_ == 1 ? 1 : 0};
        using K = detail::PullAdapter<Op>;
        const int cap = (int)kPullChunk + P_ + 2;
        const size_t smem = pull_acc_offset(cap) + sizeof(Acc) * cap + cap;
        check(cudaFuncSetAttribute(k_pull<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem");
        int per_sm = 0;
        check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pull<K>, kPullThreads, smem), "occupancy");
        const unsigned g = (unsigned)std::min<uint64_t>(sd.nchunks, (uint64_t)num_sms_ * (uint64_t)std::max(per_sm, 1));
        k_pull<K><<<g, kPullThreads, smem, stream_>>>(pa, sd.pull_adj, sd.pull_cidx, sd.pull_cvert, sd.chunk, E_,
                                                     sd.nitems, sd.nchunks, V_, cap);
        check(cudaGetLastError(), "k_pull");
        const uint64_t n = P_ == 1 ? sd.nsplit : V_;
        if (n)
            detail::k_dense_finish<Op><<<grid(n), 256, 0, stream_>>>(op, P_ == 1 ? sd.split : nullptr, sd.pull_cvert,
                                                                    sd.nsplit, sd.pull_deg, V_,
                                                                    static_cast<Acc*>(partial_), out);
        check(cudaGetLastError(), "k_dense_finish");
    }

    // master/mirror dense step: each partition reduces its in-lists per destination (a list that
    // crosses chunk boundaries gives one partial per chunk) and addresses the partial to the
    // destination's master partition; each master buffer then goes through dense_slot
    template <class Op>
    void run_dense_msgs(const Op& op, typename Op::R* out) {
        using Acc = typename Op::Acc;
        const Side& sd = *cur_;
        if (sd.nchunks == 0) return;
        if (!dbase_) setup_dense_buffers(sd);
        const uint64_t cap = h_dbase_[P_];
        if (ddata_bytes_ < sizeof(Acc) * cap) {
            if (ddata_) cudaFree(ddata_);
            ddata_ = nullptr;
            check(cudaMalloc(&ddata_, sizeof(Acc) * std::max<uint64_t>(cap, 1)), "cudaMalloc");
            ddata_bytes_ = sizeof(Acc) * cap;
        }
        check(cudaMemsetAsync(dcount_, 0, 4 * ((size_t)P_ + 1), stream_), "cudaMemsetAsync");
        int* overflow = reinterpret_cast<int*>(dcount_ + P_);
        using K = detail::PullMsgAdapter<Op>;
        K pa{op, sd.pull_w, part_off_, P_, dvert_, static_cast<Acc*>(ddata_), dbase_, dcount_, overflow};
        const int cap_items = (int)kPullChunk + P_ + 2;
        const size_t smem = pull_acc_offset(cap_items) + sizeof(Acc) * cap_items + cap_items;
        check(cudaFuncSetAttribute(k_pull<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem");
        int per_sm = 0;
        check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pull<K>, kPullThreads, smem), "occupancy");
        const unsigned g = (unsigned)std::min<uint64_t>(sd.nchunks, (uint64_t)num_sms_ * (uint64_t)std::max(per_sm, 1));
        k_pull<K><<<g, kPullThreads, smem, stream_>>>(pa, sd.pull_adj, sd.pull_cidx, sd.pull_cvert, sd.chunk, E_,
                                                     sd.nitems, sd.nchunks, V_, cap_items);
        check(cudaGetLastError(), "k_pull");
        detail::k_slot_msgs<Op><<<grid(cap), 256, 0, stream_>>>(op, dvert_, static_cast<const Acc*>(ddata_), dbase_,
                                                               dcount_, P_, out);
        check(cudaGetLastError(), "k_slot_msgs");
        std::vector<uint32_t> cnt((size_t)P_ + 1);
        check(cudaMemcpyAsync(cnt.data(), dcount_, 4 * ((size_t)P_ + 1), cudaMemcpyDeviceToHost, stream_),
              "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        if (cnt[P_]) throw Error(EG_ERR_STATE, "process_edges: a dense message buffer overflowed");
        for (int i = 0; i < P_; ++i) {
            stats_.per_partition[i] = cnt[i];
            stats_.messages += cnt[i];
        }
        stats_.bytes = stats_.messages * (sizeof(uint32_t) + sizeof(Acc));
    }

    // dense message buffers, one per master partition: capacity = the compressed entries whose
    // destination it owns (one per (source partition, destination) list) + one per chunk boundary
    void setup_dense_buffers(const Side& sd) {
        unsigned long long* d_cnt = alloc<unsigned long long>((size_t)P_);
        check(cudaMemsetAsync(d_cnt, 0, 8 * (size_t)P_, stream_), "cudaMemsetAsync");
        detail::k_items_per_owner<<<grid(sd.nitems), 256, 0, stream_>>>(sd.pull_cvert, sd.nitems, V_, part_off_, P_,
                                                                        d_cnt);
        check(cudaGetLastError(), "k_items_per_owner");
        std::vector<unsigned long long> cnt((size_t)P_);
        check(cudaMemcpyAsync(cnt.data(), d_cnt, 8 * (size_t)P_, cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        cudaFree(d_cnt);
        h_dbase_.assign((size_t)P_ + 1, 0);
        for (int i = 0; i < P_; ++i) h_dbase_[i + 1] = h_dbase_[i] + cnt[i] + sd.nchunks + 1;
        dbase_ = alloc<uint64_t>((size_t)P_ + 1);
        check(cudaMemcpyAsync(dbase_, h_dbase_.data(), 8 * ((size_t)P_ + 1), cudaMemcpyHostToDevice, stream_), "dbase");
        dvert_ = alloc<uint32_t>(std::max<uint64_t>(h_dbase_[P_], 1));
        dcount_ = alloc<uint32_t>((size_t)P_ + 1);
        check(cudaStreamSynchronize(stream_), "dbase");
    }


    void setup_pull_chunks(Side& sd) {
        sd.nchunks = (E_ + kPullChunk - 1) / kPullChunk;
        sd.chunk = alloc<uint32_t>(sd.nchunks + 2);
        sd.split = alloc<uint32_t>(sd.nchunks + 2);
        check(cudaMemsetAsync(counters_, 0, 64, stream_), "cudaMemsetAsync");
        k_pull_chunks<<<grid(sd.nitems), 256, 0, stream_>>>(sd.pull_cidx, sd.pull_cvert, sd.nitems, sd.nchunks, sd.chunk,
                                                           sd.split, counters_);
        check(cudaGetLastError(), "k_pull_chunks");
        check(cudaMemcpyAsync(&sd.nsplit, counters_, 8, cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        sd.ready = true;
    }

    void setup_transposed() {
        Side& b = side_[1];
        b.push_off = csc_.off;
        b.push_adj = csc_.adj;
        b.push_w = csc_.w;
        b.push_deg = indeg_;
        b.pull_adj = csr_.adj;
        b.pull_w = csr_.w;
        b.pull_deg = outdeg_;
        // compressed index over the CSR: one {vertex, start} per vertex with out-edges + {V, E}
        row_cvert_ = alloc<uint32_t>((size_t)V_ + 1);
        row_cidx_ = alloc<uint64_t>((size_t)V_ + 1);
        const uint64_t n = (uint64_t)V_ + 1;
        const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
        uint64_t* desc = alloc<uint64_t>(tiles);
        check(cudaMemsetAsync(desc, 0, 8 * tiles, stream_), "cudaMemsetAsync");
        check(cudaMemsetAsync(counters_ + 5, 0, 8, stream_), "cudaMemsetAsync");
        uint32_t* ticket = reinterpret_cast<uint32_t*>(counters_ + 5);
        uint64_t* total = reinterpret_cast<uint64_t*>(counters_ + 4);
        k_scan<<<(unsigned)tiles, kScanThreads, 0, stream_>>>(detail::LoadHasOut{outdeg_, V_},
                                                               detail::EpiRowIndex{csr_.off, V_, E_, row_cvert_, row_cidx_},
                                                               n, desc, ticket, reinterpret_cast<int*>(ticket + 1), total,
                                                               kLookbackSpinCap);
        check(cudaGetLastError(), "k_scan");
        unsigned long long nc = 0;
        int err = 0;
        check(cudaMemcpyAsync(&nc, total, 8, cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
        check(cudaMemcpyAsync(&err, ticket + 1, 4, cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        cudaFree(desc);
        if (err) throw Error(EG_ERR_TIMEOUT, "set_transposed: a bounded device wait gave up");
        b.pull_cvert = row_cvert_;
        b.pull_cidx = row_cidx_;
        b.nitems = nc - 1;  // the sentinel closes the last list
        setup_pull_chunks(b);
    }

    // the identity is a device function; evaluate it once on the device
    template <class Op>
    typename Op::Acc host_identity(const Op& op) {
        using Acc = typename Op::Acc;
        Acc* d = reinterpret_cast<Acc*>(counters_ + 7);
        detail::k_fill_acc<Op><<<1, 1, 0, stream_>>>(d, 1, op);
        check(cudaGetLastError(), "k_fill_acc");
        Acc h;
        check(cudaMemcpyAsync(&h, d, sizeof(Acc), cudaMemcpyDeviceToHost, stream_), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        return h;
    }

    eg_graph* g_;
    uint32_t V_ = 0;
    uint64_t E_ = 0;
    int P_ = 1;
    eg_csr_view csr_{};
    eg_csc_view csc_{};
    cudaStream_t stream_ = nullptr;
    int num_sms_ = 152;
    uint32_t* outdeg_ = nullptr;
    uint32_t* indeg_ = nullptr;
    unsigned long long* counters_ = nullptr;  // [2..3] queue length + active edges, [4] emitters, [5] scan ticket/error, [6] result, [7] identity
    uint32_t* q0_ = nullptr;
    uint32_t* q1_ = nullptr;
    uint64_t* ipref_ = nullptr;
    uint32_t* push_chunk_ = nullptr;
    uint64_t* scan_desc_ = nullptr;
    Side side_[2];  // as built, transposed
    Side* cur_ = nullptr;
    uint32_t* row_cvert_ = nullptr;
    uint64_t* row_cidx_ = nullptr;
    void* msg_ = nullptr;
    size_t msg_bytes_ = 0;
    void* partial_ = nullptr;
    size_t partial_bytes_ = 0, partial_size_ = 0;
    unsigned long long partial_id_ = 0;
    bool last_dense_ = false;
    uint64_t last_active_edges_ = 0;
    // master/mirror message path
    bool msg_path_ = false;
    std::vector<uint32_t> h_part_off_;
    uint32_t* part_off_ = nullptr;
    uint32_t* mvert_ = nullptr;   // sparse buffers: partition p's messages start at part_off[p]
    void* mdata_ = nullptr;
    size_t mdata_bytes_ = 0;
    uint32_t* mcount_ = nullptr;
    uint32_t* dvert_ = nullptr;   // dense buffers: master partition i's messages start at dbase[i]
    void* ddata_ = nullptr;
    size_t ddata_bytes_ = 0;
    uint64_t* dbase_ = nullptr;
    std::vector<uint64_t> h_dbase_;
    uint32_t* dcount_ = nullptr;  // [P] message counts, [P] overflow flag
    MessageStats stats_;
};

}  // namespace engine
}  // namespace eg
