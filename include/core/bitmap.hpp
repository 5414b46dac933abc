// bitmap.hpp — VertexSubset of the Graph<EdgeData> API: one bit per vertex in 64-bit words,
// the word/bit split of the reference's BitmapType (core/bitmap.hpp:20-68).  The words live in
// host memory that the GPU of a GB300 node can also read (ordinary allocation; the engine copies
// a subset to the device when it needs one).
#ifndef EG_CORE_BITMAP_HPP
#define EG_CORE_BITMAP_HPP

#include <stddef.h>
#include <string.h>

#define WORD_OFFSET(i) ((i) >> 6)
#define BIT_OFFSET(i) ((i) & 0x3f)

class BitmapType {
   public:
    size_t size;
    unsigned long* data;

    BitmapType() : size(0), data(nullptr) {}
    explicit BitmapType(size_t n) : size(n), data(new unsigned long[WORD_OFFSET(n) + 1]) { clear(); }
    ~BitmapType() { delete[] data; }
    BitmapType(const BitmapType&) = delete;
    BitmapType& operator=(const BitmapType&) = delete;

    size_t words() const { return WORD_OFFSET(size) + 1; }
    void clear() { memset(data, 0, sizeof(unsigned long) * words()); }
    // every vertex in [0, size) set, nothing beyond
    void fill() {
        const size_t full = WORD_OFFSET(size);
        for (size_t w = 0; w < full; ++w) data[w] = ~0ul;
        const size_t rem = BIT_OFFSET(size);
        data[full] = rem ? ((1ul << rem) - 1ul) : 0ul;
    }
    unsigned long get_bit(size_t i) const { return data[WORD_OFFSET(i)] & (1ul << BIT_OFFSET(i)); }
    void set_bit(size_t i) { __atomic_fetch_or(data + WORD_OFFSET(i), 1ul << BIT_OFFSET(i), __ATOMIC_RELAXED); }
};

typedef BitmapType VertexSubset;

#endif
