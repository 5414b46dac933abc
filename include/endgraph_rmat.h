/*
 * endgraph_rmat.h — seeded, counter-based R-MAT edge generator.
 *
 * The reference ships no generator (it reads a binary edge file, core/graph.hpp:1011-1084,
 * records laid out as core/type.hpp:29-43).  This header defines the synthetic inputs every
 * test and benchmark of this project uses.  Edge i is a pure function of (params, i), so the
 * CUDA generator (endgraph_gb300/csrc/eg_generate.cu) and any host code produce identical
 * edge lists, in the same order, without sharing state.
 *
 * Per edge: `scale` quadrant draws (a -> (0,0), b -> (0,1), c -> (1,0), d -> (1,1)), MSB first,
 * each from one 32-bit word compared with integer thresholds; an edge with an endpoint >= V is
 * redrawn (at most 64 attempts, then reduced mod V).  Vertex ids are then optionally relabelled
 * by a seeded bijection of [0, V) (multiply/xorshift rounds on `scale` bits + cycle walking).
 * Weights are w = fmaf(w_hi - w_lo, u24 * 2^-24, w_lo) from an independent draw.
 * Random words come from the SplitMix64 output function (Steele, Lea, Flood, OOPSLA 2014).
 */
#ifndef ENDGRAPH_RMAT_H
#define ENDGRAPH_RMAT_H

#include <stdint.h>
#include <math.h>

#ifdef __CUDACC__
#define EG_HD __host__ __device__ __forceinline__
#else
#define EG_HD static inline
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct eg_rmat_params {
    uint64_t seed;
    uint64_t E;          /* number of edges */
    uint32_t V;          /* vertex ids are < V */
    uint32_t scale;      /* 2^scale >= V */
    uint32_t ta;         /* floor(a * 2^32) */
    uint32_t tab;        /* floor((a+b) * 2^32) */
    uint32_t tabc;       /* floor((a+b+c) * 2^32) */
    uint32_t permute;    /* 1: relabel ids by a seeded bijection of [0, V) */
    float w_lo, w_hi;    /* weights uniform in [w_lo, w_hi) */
} eg_rmat_params;

EG_HD uint64_t eg_mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* j-th 32-bit word of the stream keyed by `base` */
EG_HD uint32_t eg_rmat_word(uint64_t base, uint32_t j) {
    uint64_t r = eg_mix64(base + (uint64_t)(j >> 1));
    return (uint32_t)(r >> ((j & 1u) * 32u));
}

/* one bijective round on [0, 2^scale) */
EG_HD uint32_t eg_perm_round(uint32_t x, uint32_t mask, uint32_t shift, uint64_t key) {
    x = (x * ((uint32_t)key | 1u)) & mask;
    x ^= x >> shift;
    x = (x + (uint32_t)(key >> 32)) & mask;
    return x;
}

/* seeded bijection of [0, V); x < V */
EG_HD uint32_t eg_permute_vertex(uint32_t x, uint32_t V, uint32_t scale, uint64_t seed) {
    uint32_t mask = scale >= 32 ? 0xFFFFFFFFu : ((1u << scale) - 1u);
    uint32_t shift = scale / 2u > 0u ? scale / 2u : 1u;
    uint64_t k0 = eg_mix64(seed ^ 0xA0761D6478BD642Full);
    uint64_t k1 = eg_mix64(k0), k2 = eg_mix64(k1), k3 = eg_mix64(k2);
    do {
        x = eg_perm_round(x, mask, shift, k0);
        x = eg_perm_round(x, mask, shift, k1);
        x = eg_perm_round(x, mask, shift, k2);
        x = eg_perm_round(x, mask, shift, k3);
    } while (x >= V);
    return x;
}

/* edge i of the R-MAT stream */
EG_HD void eg_rmat_edge(const eg_rmat_params* p, uint64_t i, uint32_t* src, uint32_t* dst, float* w) {
    uint64_t base = eg_mix64(p->seed * 0x9E3779B97F4A7C15ull + i);
    uint32_t s = 0, d = 0;
    for (uint32_t attempt = 0; attempt < 64u; ++attempt) {
        s = 0; d = 0;
        for (uint32_t l = 0; l < p->scale; ++l) {
            uint32_t u = eg_rmat_word(base, attempt * p->scale + l);
            uint32_t sb = 0, db = 0;
            if (u < p->ta) { sb = 0; db = 0; }
            else if (u < p->tab) { sb = 0; db = 1; }
            else if (u < p->tabc) { sb = 1; db = 0; }
            else { sb = 1; db = 1; }
            s = (s << 1) | sb;
            d = (d << 1) | db;
        }
        if (s < p->V && d < p->V) break;
        if (attempt == 63u) { s %= p->V; d %= p->V; }
    }
    if (p->permute) {
        uint64_t pseed = p->seed ^ 0x5851F42D4C957F2Dull;
        s = eg_permute_vertex(s, p->V, p->scale, pseed);
        d = eg_permute_vertex(d, p->V, p->scale, pseed);
    }
    *src = s;
    *dst = d;
    if (w) {
        uint32_t u = (uint32_t)eg_mix64(base ^ 0xD1B54A32D192ED03ull);
        float x = (float)(u >> 8) * 5.9604644775390625e-08f; /* 2^-24 */
        *w = fmaf(p->w_hi - p->w_lo, x, p->w_lo);
    }
}

/* fill the params struct from probabilities (host side) */
static inline void eg_rmat_init(eg_rmat_params* p, uint32_t V, uint64_t E, double a, double b, double c,
                                uint64_t seed, uint32_t permute, float w_lo, float w_hi) {
    uint32_t scale = 0;
    while (scale < 32u && ((uint64_t)1 << scale) < (uint64_t)V) ++scale;
    p->seed = seed; p->E = E; p->V = V; p->scale = scale;
    p->ta = (uint32_t)(a * 4294967296.0);
    p->tab = (uint32_t)((a + b) * 4294967296.0);
    p->tabc = (uint32_t)((a + b + c) * 4294967296.0);
    p->permute = permute; p->w_lo = w_lo; p->w_hi = w_hi;
}

#ifdef __cplusplus
}
#endif

#endif /* ENDGRAPH_RMAT_H */
