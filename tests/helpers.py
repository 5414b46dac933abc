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
