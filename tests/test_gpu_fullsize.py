"""Parity at full size: the GPU build and toolkits against the reference's own engine (oracle/_ref,
core/graph.hpp compiled at one rank) on the same seeded graphs as the benchmark.

* The bench workload: R-MAT with 2^25 vertices and 2^29 edges, ids permuted -- degrees, the CPBT
  partition, the CSR (index at every source, source bitmap, per-list neighbour signatures), the
  CSC (compressed index, per-list signatures), PageRank x20 (FP32 against the reference's FP64,
  relative L1 <= 1e-6) and BFS levels from the bench's 16 roots (bit-exact, parents a BFS tree).
* A power-law stand-in for the twitter-2010-sized configuration at 2^24 vertices and 2^29
  weighted edges: SSSP distances bit-exact, and CC labels bit-exact on the symmetrised graph
  (2^30 edges).

Per-list signatures are sums of a 64-bit mix of each neighbour (and weight bits), so they compare
whole lists without depending on the order inside a list, which the reference leaves to its
threads.  Each comparison runs outside any timing; the reference takes tens of seconds per graph
on the host cores."""
import os

import numpy as np
import pytest

import oracle
from helpers import rel_l1

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not oracle.Reference.available(),
                                 reason="reference engine (oracle/_ref) not built on this machine")]

SEED = 20240601  # the bench's seed


def _host_gib():
    try:
        return os.sysconf("SC_PHYS_PAGES") * os.sysconf("SC_PAGE_SIZE") / 2**30
    except (ValueError, OSError):
        return 0.0


def _bits(words, V):
    return np.unpackbits(np.ascontiguousarray(words).view(np.uint8), bitorder="little")[:V].astype(bool)


def _bench_roots(src, E, seed, n):
    """The bench's roots: sources of 64 edges drawn by torch's seeded CPU generator."""
    import torch
    gen = torch.Generator(device="cpu").manual_seed(seed)
    ridx = torch.randint(0, E, (64,), generator=gen).numpy()
    return [int(src[i]) for i in ridx[:n]]


def test_bench_workload_matches_reference(eg_lib):
    import endgraph_gb300 as eg
    if _host_gib() < 48:
        pytest.skip(f"needs about 40 GiB of host memory for the reference run ({_host_gib():.0f} GiB here)")
    V, E = 1 << 25, 1 << 29
    src, dst, _ = oracle.rmat(V, E, SEED, permute=True)
    R = oracle.Reference(src, dst, None, V, eta=1, max_iterations=20)
    R.build()
    ref = R.summary()
    with eg.Graph(eta=1, max_iterations=20) as g:
        rec = eg.pack_edges(src, dst)
        g.load_directed(rec, V)
        del rec
        outd, ind = g.degrees()
        assert np.array_equal(outd, ref["degree"])  # dense mode: the reference keeps out-degrees
        assert int(ind.sum()) == E
        po, _ = g.partition()
        assert np.array_equal(po, ref["partition_offset"])
        csr = g.csr()
        assert np.array_equal(csr["bitmap"][0], ref["csr_bitmap"])
        # the reference's outgoing_adj_index is written at each source and one past it
        sv = np.nonzero(_bits(ref["csr_bitmap"], V))[0]
        off = csr["off"][0]
        assert np.array_equal(off[sv], ref["csr_index"][sv])
        assert np.array_equal(off[sv + 1], ref["csr_index"][sv + 1])
        assert np.array_equal(np.diff(off.astype(np.int64)), outd.astype(np.int64))
        assert np.array_equal(oracle.list_hash(off, csr["adj"]), ref["hout"])
        csc = g.csc()
        assert np.array_equal(csc["cvert"], ref["cvert"])
        assert np.array_equal(csc["cidx"], ref["cidx"])
        assert np.array_equal(oracle.list_hash(csc["off"][0], csc["adj"]), ref["hin"])
        del csc
        # PageRank x20: FP32 ranks against the reference's FP64 run
        pr = g.pagerank(20, 0.85)
        ref_pr, _ = R.pagerank(20)
        err = rel_l1(pr, ref_pr)
        print(f"PageRank 2^25/2^29: FP32 relative L1 against the reference's FP64 = {err:.3e}")
        assert err <= 1e-6, err
        # BFS from the bench's 16 roots
        for r in _bench_roots(src, E, SEED, 16):
            lv, par = g.bfs(r)
            ref_lv, _, _ = R.bfs(r)
            assert np.array_equal(lv, ref_lv), r
            assert oracle.bfs_check_parents(off, csr["adj"], V, r, lv, par) == 0, r
    R.close()


def test_power_law_stand_in_matches_reference(eg_lib):
    import endgraph_gb300 as eg
    if _host_gib() < 64:
        pytest.skip(f"needs about 50 GiB of host memory for the reference runs ({_host_gib():.0f} GiB here)")
    V, E = 1 << 24, 1 << 29
    src, dst, w = oracle.rmat(V, E, SEED + 21, permute=True, weights=(0.0, 1.0))
    outd, _ = oracle.degrees(src, dst, V)
    cand = src[np.arange(0, E, E // 64)]
    root = int(cand[0])
    # SSSP on the weighted directed graph
    R = oracle.Reference(src, dst, w, V, eta=1, max_iterations=20)
    R.build()
    ref_dist, _ = R.sssp(root)
    R.close()
    with eg.Graph(eta=1, max_iterations=20) as g:
        rec = eg.pack_edges(src, dst, w)
        g.load_directed(rec, V)
        del rec
        dist = g.sssp(root)
    assert np.array_equal(dist.view(np.uint32), ref_dist.view(np.uint32))
    print(f"SSSP 2^24/2^29 weighted: {int((ref_dist < 1e9).sum())} reached, max out-degree {int(outd.max())}")
    del w
    # CC on the symmetrised graph (load_undirected_from_directed: 2^30 edges)
    R = oracle.Reference(src, dst, None, V, symmetric=True, eta=1, max_iterations=20)
    R.build()
    ref_label, iters, _ = R.cc()
    R.close()
    with eg.Graph(eta=1, max_iterations=20) as g:
        rec = eg.pack_edges(src, dst)
        g.load_undirected_from_directed(rec, V)
        del rec
        label = g.cc()
    assert np.array_equal(label, ref_label)
    print(f"CC 2^24/2^30 symmetrised: {int((ref_label == np.arange(V)).sum())} components, "
          f"{iters} reference iterations")
