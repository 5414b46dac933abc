"""Shared helpers for the parity tests: seeded graphs and order-independent comparisons."""
import numpy as np

import oracle

RMAT = dict(a=0.57, b=0.19, c=0.19)


def rmat_graph(V, E, seed, permute=True, weights=None):
    src, dst, w = oracle.rmat(V, E, seed, permute=permute, weights=weights, **RMAT)
    return src, dst, w


def lists_equal(off_a, adj_a, off_b, adj_b, w_a=None, w_b=None):
    """Same offsets and, per list, the same multiset of (neighbour, weight)."""
    off_a = np.asarray(off_a, np.uint64)
    off_b = np.asarray(off_b, np.uint64)
    if not np.array_equal(off_a, off_b):
        return False
    a, wa = oracle.sorted_lists(off_a, adj_a, w_a)
    b, wb = oracle.sorted_lists(off_b, adj_b, w_b)
    if not np.array_equal(a, b):
        return False
    if wa is not None or wb is not None:
        return np.array_equal(wa.view(np.uint32), wb.view(np.uint32))
    return True


def rel_l1(x, ref):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.abs(x - ref).sum() / max(np.abs(ref).sum(), 1e-300))


def graph_batch(G, seed, weighted=False):
    """G small R-MAT graphs (V log-uniform in [100, 5000], edge factor 4..32) back to back: vertex
    counts, record offsets, the per-graph (src, dst, w) and the concatenated lists."""
    rng = np.random.default_rng(seed)
    Vs = np.exp(rng.uniform(np.log(100), np.log(5000), G)).astype(np.uint32)
    efs = rng.integers(4, 33, G)
    parts = []
    for i in range(G):
        s, d, w = rmat_graph(int(Vs[i]), int(Vs[i] * efs[i]), seed * 1000 + i, weights=(0.0, 1.0) if weighted else None)
        parts.append((s, d, w))
    eoff = np.zeros(G + 1, np.uint64)
    eoff[1:] = np.cumsum([len(p[0]) for p in parts])
    src = np.concatenate([p[0] for p in parts])
    dst = np.concatenate([p[1] for p in parts])
    w = np.concatenate([p[2] for p in parts]) if weighted else None
    return Vs, eoff, parts, src, dst, w
