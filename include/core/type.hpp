// type.hpp — edge record and adjacency types of the Graph<EdgeData> API.
// The records must keep the reference's binary layout (core/type.hpp:23-74 of leodestiny/EndGraph):
// edge files are read as packed {u32 src, u32 dst[, EdgeData]} records, so the same structs are
// declared here with the same field names and packing.
#ifndef EG_CORE_TYPE_HPP
#define EG_CORE_TYPE_HPP

#include <stdint.h>

struct Empty {};

typedef uint32_t UINT;
typedef uint64_t ULLONG;

template <typename EdgeData>
struct EdgeType {
    UINT src;
    UINT dst;
    EdgeData edge_data;
} __attribute__((packed));

template <>
struct EdgeType<Empty> {
    UINT src;
    union {
        UINT dst;
        Empty edge_data;
    };
} __attribute__((packed));

template <typename EdgeData>
struct AdjacentType {
    UINT neighbour;
    EdgeData edge_data;
} __attribute__((packed));

template <>
struct AdjacentType<Empty> {
    union {
        UINT neighbour;
        Empty edge_data;
    };
} __attribute__((packed));

struct CompressedAdjIndexType {
    ULLONG index;
    UINT vertex;
    CompressedAdjIndexType() {}
    CompressedAdjIndexType(ULLONG i, UINT v) : index(i), vertex(v) {}
} __attribute__((packed));

template <typename EdgeData>
struct AdjacentListType {
    EdgeType<EdgeData>* begin;
    EdgeType<EdgeData>* end;
    AdjacentListType() : begin(nullptr), end(nullptr) {}
    AdjacentListType(EdgeType<EdgeData>* b, EdgeType<EdgeData>* e) : begin(b), end(e) {}
};

static_assert(sizeof(EdgeType<Empty>) == 8, "edge record layout");
static_assert(sizeof(EdgeType<float>) == 12, "weighted edge record layout");
static_assert(sizeof(CompressedAdjIndexType) == 12, "compressed index layout");

#endif
