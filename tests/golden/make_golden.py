"""Regenerates tests/golden/*.npz from the reference's own engine (oracle/_ref/libeg_ref.so, built
from the reference sources at one rank).  Run from the repository root:

    python tests/golden/make_golden.py

Each fixture holds a seeded R-MAT input (stored as its generator parameters and the edge arrays) and
the reference's outputs on it: CPBT partition boundaries for several partition counts, the CSR and
CSC structures (lists sorted per vertex), the compressed incoming index, PageRank (FP64, 20
iterations), BFS levels/parents, CC labels and SSSP distances.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def sorted_by_list(src, dst, w, V, key_src):
    """(offsets, neighbours, weights) with each list sorted by neighbour then weight bits."""
    key = src if key_src else dst
    other = dst if key_src else src
    cols = [other.astype(np.int64), key.astype(np.int64)]
    if w is not None:
        cols.insert(0, w.view(np.uint32).astype(np.int64))
    order = np.lexsort(tuple(cols))
    off = np.zeros(V + 1, np.uint64)
    np.cumsum(np.bincount(key, minlength=V), out=off[1:])
    return off, other[order], (None if w is None else w[order])


def make(name, V, E, seed, weighted, parts=(1, 2, 3, 4, 8)):
    weights = (0.0, 1.0) if weighted else None
    src, dst, w = oracle.rmat(V, E, seed, weights=weights)
    d = dict(V=np.uint32(V), E=np.uint64(E), seed=np.uint64(seed), src=src, dst=dst)
    if weighted:
        d["w"] = w
    # CPBT for several partition counts, both histogram modes, eta 1 and 5, two sockets
    for P in parts:
        for dense in (True, False):
            for eta in (1, 5):
                po, lo, deg = oracle.Reference.cpbt(src, dst, V, P, S=2, eta=eta, max_iterations=20, dense=dense)
                d[f"cpbt_P{P}_{'dense' if dense else 'sparse'}_eta{eta}"] = po
                d[f"cpbt_local_P{P}_{'dense' if dense else 'sparse'}_eta{eta}"] = lo
    R = oracle.Reference(src, dst, w, V)
    R.build()
    s = R.structure()
    d["degree_out"] = s["degree"]
    off, adj, ww = sorted_by_list(s["csr_src"], s["csr_dst"], s["csr_w"], V, True)
    d["csr_off"], d["csr_adj"] = off, adj
    off, adj, ww2 = sorted_by_list(s["csc_src"], s["csc_dst"], s["csc_w"], V, False)
    d["csc_off"], d["csc_adj"] = off, adj
    if weighted:
        d["csr_w"], d["csc_w"] = ww, ww2
    d["cvert"], d["cidx"] = s["cvert"], s["cidx"]
    roots = np.array([src[0], src[len(src) // 3], dst[5]], np.uint32)
    d["roots"] = roots
    if not weighted:
        pr, _ = R.pagerank(20)
        d["pagerank20"] = pr
        for i, r in enumerate(roots):
            lv, par, _ = R.bfs(int(r))
            d[f"bfs_level_{i}"] = lv
            d[f"bfs_parent_{i}"] = par
    else:
        for i, r in enumerate(roots):
            dist, _ = R.sssp(int(r))
            d[f"sssp_{i}"] = dist
    R.close()
    if not weighted:
        RS = oracle.Reference(src, dst, None, V, symmetric=True)
        RS.build()
        lab, iters, _ = RS.cc()
        d["cc_label"] = lab
        d["cc_iterations"] = np.int32(iters)
        RS.close()
    path = os.path.join(OUT, f"{name}.npz")
    np.savez_compressed(path, **d)
    print(path, os.path.getsize(path))


def main():
    if not oracle.Reference.available() and oracle.build_ref() is None:
        raise SystemExit("reference engine unavailable: build oracle/_ref first")
    # optimal_offset known answers (the reference's own function)
    kat = {}
    a = np.array([5, 0, 0, 7, 1, 0, 9, 3, 0, 2], np.uint64)
    for k in (1, 2, 3, 4, 5, 10, 11):
        kat[f"kat_a_k{k}"] = oracle.Reference.optimal_offset(a, k)
    kat["kat_a"] = a
    z = np.zeros(4, np.uint64)
    kat["kat_zero_k3"] = oracle.Reference.optimal_offset(z, 3)
    rng = np.random.default_rng(7)
    r = (rng.integers(0, 1 << 40, 1000, dtype=np.uint64) * (rng.random(1000) < 0.7)).astype(np.uint64)
    kat["kat_rand"] = r
    for k in (1, 2, 7, 64):
        kat[f"kat_rand_k{k}"] = oracle.Reference.optimal_offset(r, k)
    np.savez_compressed(os.path.join(OUT, "optimal_offset.npz"), **kat)
    # CPBT on a graph with many pages: only the generator parameters and the boundaries are stored
    V, E, seed = 200_000, 1_000_000, 21
    src, dst, _ = oracle.rmat(V, E, seed)
    cp = dict(V=np.uint32(V), E=np.uint64(E), seed=np.uint64(seed))
    for P in (1, 2, 3, 4, 8, 16, 64):
        for S in (1, 3):
            for dense in (True, False):
                for eta in (1, 7):
                    po, lo, _ = oracle.Reference.cpbt(src, dst, V, P, S=S, eta=eta, max_iterations=20, dense=dense)
                    tag = f"P{P}_S{S}_{'dense' if dense else 'sparse'}_eta{eta}"
                    cp[f"part_{tag}"] = po
                    cp[f"local_{tag}"] = lo
    np.savez_compressed(os.path.join(OUT, "cpbt_v200000_e1000000.npz"), **cp)
    make("rmat_v4096_e16384", 4096, 16384, 11, weighted=False)
    make("rmat_v9000_e40000", 9000, 40000, 12, weighted=False, parts=(1, 2, 3))
    make("rmat_w_v5000_e20000", 5000, 20000, 13, weighted=True, parts=(1, 2))


if __name__ == "__main__":
    main()
