"""GPU parity: libendgraph_gb300 (through its C ABI) against the CPU oracle on seeded R-MAT graphs."""
import numpy as np
import pytest

import oracle
from helpers import lists_equal, rel_l1, rmat_graph

pytestmark = pytest.mark.gpu

CASES = [  # (V, E, seed)
    (1 << 12, 1 << 16, 1),
    (1 << 16, 1 << 20, 2),
    (100_000, 300_000, 3),   # V not a page multiple
    (5000, 30_000, 4),
]


def _graph(eg_lib, P=1, S=1, eta=1, T=20):
    import endgraph_gb300 as eg
    return eg.Graph(eta=eta, partitions=P, sub_partitions=S, max_iterations=T)


@pytest.mark.parametrize("V,E,seed", CASES)
def test_structure_single_partition(eg_lib, V, E, seed):
    import endgraph_gb300 as eg
    src, dst, _ = rmat_graph(V, E, seed)
    with _graph(eg_lib) as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        outd, ind = g.degrees()
        o_out, o_in = oracle.degrees(src, dst, V)
        assert np.array_equal(outd, o_out) and np.array_equal(ind, o_in)
        po, lo = g.partition()
        opo, olo = oracle.cpbt(o_out, V, 1, 1, 1, 20, True)
        assert np.array_equal(po, opo) and np.array_equal(lo, olo)
        ref_csr = oracle.build_csr(src, dst, None, V, opo)
        ref_csc = oracle.build_csc(src, dst, None, V, opo)
        csr = g.csr()
        csc = g.csc()
        assert lists_equal(csr["off"][0], csr["adj"], ref_csr["off"][0], ref_csr["adj"])
        assert np.array_equal(csr["bitmap"], ref_csr["bitmap"])
        assert lists_equal(csc["off"][0], csc["adj"], ref_csc["off"][0], ref_csc["adj"])
        assert np.array_equal(csc["cvert"], ref_csc["cvert"])
        assert np.array_equal(csc["cidx"], ref_csc["cidx"])


@pytest.mark.parametrize("P,S", [(2, 1), (3, 2), (8, 3), (16, 1)])
def test_structure_partitions(eg_lib, P, S):
    import endgraph_gb300 as eg
    V, E = 1 << 16, 1 << 19
    src, dst, w = rmat_graph(V, E, 11 + P, weights=(0.0, 1.0))
    with _graph(eg_lib, P=P, S=S, eta=3) as g:
        g.load_directed(eg.pack_edges(src, dst, w), V)
        o_out, _ = oracle.degrees(src, dst, V)
        opo, olo = oracle.cpbt(o_out, V, P, S, 3, 20, True)
        po, lo = g.partition()
        assert np.array_equal(po, opo) and np.array_equal(lo, olo)
        ref_csr = oracle.build_csr(src, dst, w, V, opo)
        ref_csc = oracle.build_csc(src, dst, w, V, opo)
        csr, csc = g.csr(), g.csc()
        for p in range(P):
            assert lists_equal(csr["off"][p], csr["adj"], ref_csr["off"][p], ref_csr["adj"], csr["w"], ref_csr["w"])
            assert lists_equal(csc["off"][p], csc["adj"], ref_csc["off"][p], ref_csc["adj"], csc["w"], ref_csc["w"])
        assert np.array_equal(csr["bitmap"], ref_csr["bitmap"])
        assert np.array_equal(csc["cvert"], ref_csc["cvert"])
        assert np.array_equal(csc["cidx"], ref_csc["cidx"])


@pytest.mark.parametrize("V,E,seed", CASES)
@pytest.mark.parametrize("P", [1, 3])
def test_pagerank(eg_lib, V, E, seed, P):
    import endgraph_gb300 as eg
    src, dst, _ = rmat_graph(V, E, seed)
    o_out, _ = oracle.degrees(src, dst, V)
    csc = oracle.build_csc(src, dst, None, V, np.array([0, V], np.uint32))
    ref = oracle.pagerank(csc["off"][0], csc["adj"], o_out, V, 20, 0.85)
    with _graph(eg_lib, P=P) as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        pr = g.pagerank(20, 0.85)
    err = rel_l1(pr, ref)
    assert err <= 1e-6, err


@pytest.mark.parametrize("P", [1, 3])
def test_pagerank_renumbered_gathers(eg_lib, P):
    """Gathering through sources renumbered by out-degree class sums the same values: the ranks
    match the vertex-order run for 0, 1, 2 and 20 iterations (up to the order of the float
    additions, which the shared-memory partial sums leave open in both), and a rebuild renumbers
    again."""
    import endgraph_gb300 as eg
    V, E = 50_000, 600_000
    src, dst, _ = rmat_graph(V, E, 77)
    o_out, _ = oracle.degrees(src, dst, V)
    csc = oracle.build_csc(src, dst, None, V, np.array([0, V], np.uint32))
    with _graph(eg_lib, P=P) as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        for iters in (0, 1, 2, 20):
            g.set_option(eg.EG_OPT_PR_RELABEL, 0)
            plain = g.pagerank(iters, 0.85)
            g.set_option(eg.EG_OPT_PR_RELABEL, 1)
            ren = g.pagerank(iters, 0.85)
            assert rel_l1(ren, plain) <= 1e-6, iters
        ref = oracle.pagerank(csc["off"][0], csc["adj"], o_out, V, 20, 0.85)
        assert rel_l1(ren, ref) <= 1e-6
        # a second graph on the same handle: the renumbering follows the new degrees
        src2, dst2, _ = rmat_graph(V, E // 2, 78)
        g.load_directed(eg.pack_edges(src2, dst2), V)
        o2, _ = oracle.degrees(src2, dst2, V)
        csc2 = oracle.build_csc(src2, dst2, None, V, np.array([0, V], np.uint32))
        ref2 = oracle.pagerank(csc2["off"][0], csc2["adj"], o2, V, 20, 0.85)
        assert rel_l1(g.pagerank(20, 0.85), ref2) <= 1e-6


def _in_degree_graph(indeg, V, seed):
    """Edges whose destinations 0..len(indeg)-1 have the given in-degrees, from random sources."""
    rng = np.random.default_rng(seed)
    dst = np.repeat(np.arange(len(indeg), dtype=np.uint32), indeg)
    src = rng.integers(0, V, len(dst), dtype=np.uint32)
    perm = rng.permutation(len(dst))
    return src[perm], dst[perm]


@pytest.mark.parametrize("shape", ["hub", "degree1", "degree16", "degree4096", "tiny", "ragged"])
def test_pagerank_chunk_shapes(eg_lib, shape):
    """The one-partition sweep cuts the CSC into 4,096-edge CTA chunks of 16-edge threads: in-lists
    that span chunks (a 9,000-edge hub), chunks of 4,096 one-edge lists, lists that end exactly on
    thread and chunk boundaries, fewer edges than one chunk, and a ragged last chunk all match the
    oracle, with and without renumbered gathers."""
    import endgraph_gb300 as eg
    V = 4096
    rng = np.random.default_rng(5)
    indeg = {
        "hub": np.concatenate([[9000], rng.integers(1, 40, 600), [1300], rng.integers(0, 3, 500)]),
        "degree1": np.ones(4096 * 2 + 100, np.int64)[:V],
        "degree16": np.full(700, 16),
        "degree4096": np.full(3, 4096),
        "tiny": np.array([1, 0, 3, 2]),
        "ragged": np.concatenate([rng.integers(1, 30, 400), [17]]),
    }[shape]
    src, dst = _in_degree_graph(indeg, V, 7)
    o_out, _ = oracle.degrees(src, dst, V)
    csc = oracle.build_csc(src, dst, None, V, np.array([0, V], np.uint32))
    ref = oracle.pagerank(csc["off"][0], csc["adj"], o_out, V, 20, 0.85)
    with _graph(eg_lib) as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        for relabel in (0, 1):
            g.set_option(eg.EG_OPT_PR_RELABEL, relabel)
            err = rel_l1(g.pagerank(20, 0.85), ref)
            assert err <= 1e-6, (relabel, err)


@pytest.mark.parametrize("V,E,seed", CASES)
@pytest.mark.parametrize("P", [1, 2])
def test_bfs(eg_lib, V, E, seed, P):
    import endgraph_gb300 as eg
    src, dst, _ = rmat_graph(V, E, seed)
    csr = oracle.build_csr(src, dst, None, V, np.array([0, V], np.uint32))
    with _graph(eg_lib, P=P) as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        for root in [int(src[0]), int(src[len(src) // 2]), 0]:
            lv_ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, root)
            lv, par = g.bfs(root)
            assert np.array_equal(lv, lv_ref)
            assert oracle.bfs_check_parents(csr["off"][0], csr["adj"], V, root, lv, par) == 0


@pytest.mark.parametrize("direction", [0, 1, 2])
@pytest.mark.parametrize("P", [1, 2])
def test_bfs_directions(eg_lib, direction, P):
    """Push-only (the reference's use_root mode), pull-only and Gemini's switch give the same levels."""
    import endgraph_gb300 as eg
    V, E = 1 << 16, 1 << 20
    src, dst, _ = rmat_graph(V, E, 77)
    csr = oracle.build_csr(src, dst, None, V, np.array([0, V], np.uint32))
    with _graph(eg_lib, P=P) as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        g.set_option(eg.EG_OPT_BFS_DIRECTION, direction)
        for root in [int(src[3]), int(dst[5])]:
            lv_ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, root)
            lv, par = g.bfs(root)
            assert np.array_equal(lv, lv_ref)
            assert oracle.bfs_check_parents(csr["off"][0], csr["adj"], V, root, lv, par) == 0
            run = g.last_run()
            reach_edges = int(np.asarray(np.diff(csr["off"][0].astype(np.int64)))[lv_ref != oracle.UNREACHED].sum())
            assert run["edges"] == reach_edges
            if direction == 1:
                assert run["pull"] == 0
            if direction == 2:
                assert run["push"] == 0


@pytest.mark.parametrize("P", [1, 2])
def test_bfs_graph_replay(eg_lib, P):
    """Single-root BFS replayed as one CUDA graph (a WHILE conditional node over the levels, the
    push/pull choice made on the device by IF conditional nodes) gives the oracle's levels and
    valid parents in every direction mode, for several roots on one captured graph and after a
    rebuild, and takes both directions as the host loop does."""
    import endgraph_gb300 as eg
    V, E = 1 << 16, 1 << 20
    src, dst, _ = rmat_graph(V, E, 5)
    csr = oracle.build_csr(src, dst, None, V, np.array([0, V], np.uint32))
    with _graph(eg_lib, P=P) as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        g.set_option(eg.EG_OPT_CUDA_GRAPH, 2)
        for direction in (0, 1, 2):
            g.set_option(eg.EG_OPT_BFS_DIRECTION, direction)
            for root in (int(src[0]), int(src[100]), 12345):
                lv, par = g.bfs(root)
                ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, root)
                assert np.array_equal(lv, ref), (direction, root)
                assert oracle.bfs_check_parents(csr["off"][0], csr["adj"], V, root, lv, par) == 0
                run = g.last_run()
                if direction == 0 and ref[ref != oracle.UNREACHED].max() > 2:
                    assert run["push"] > 0 and run["pull"] > 0
        # a rebuild (other buffers) captures a new graph
        src2, dst2, _ = rmat_graph(V, E // 2, 6)
        g.load_directed(eg.pack_edges(src2, dst2), V)
        csr2 = oracle.build_csr(src2, dst2, None, V, np.array([0, V], np.uint32))
        g.set_option(eg.EG_OPT_BFS_DIRECTION, 0)
        lv, _ = g.bfs(int(src2[0]))
        assert np.array_equal(lv, oracle.bfs_levels(csr2["off"][0], csr2["adj"], V, int(src2[0])))


def test_bfs_graph_replay_deeper_than_one_replay(eg_lib):
    """A chain of 5,000 vertices: the replay stops at its level cap (4,096) and the host loop
    finishes the traversal from the state it left."""
    import endgraph_gb300 as eg
    n = 5000
    rng = np.random.default_rng(3)
    perm = rng.permutation(n).astype(np.uint32)
    src, dst = perm[:-1], perm[1:]
    with _graph(eg_lib) as g:
        g.load_directed(eg.pack_edges(src, dst), n)
        g.set_option(eg.EG_OPT_CUDA_GRAPH, 3)
        lv, par = g.bfs(int(perm[0]))
    want = np.empty(n, np.uint32)
    want[perm] = np.arange(n, dtype=np.uint32)
    assert np.array_equal(lv, want)
    assert np.array_equal(par[perm[1:]], perm[:-1])


@pytest.mark.parametrize("V,E,seed", CASES)
def test_cc(eg_lib, V, E, seed):
    import endgraph_gb300 as eg
    src, dst, _ = rmat_graph(V, E, seed)
    ref = oracle.cc_labels(src, dst, V)
    with _graph(eg_lib) as g:
        g.load_undirected_from_directed(eg.pack_edges(src, dst), V)
        lab = g.cc()
        assert np.array_equal(lab, ref)


@pytest.mark.parametrize("V,E,seed", CASES)
@pytest.mark.parametrize("delta", [-1, 0, 50_000])  # automatic near/far step, plain sweeps, 0.05
def test_sssp(eg_lib, V, E, seed, delta):
    import endgraph_gb300 as eg
    src, dst, w = rmat_graph(V, E, seed, weights=(0.0, 1.0))
    csr = oracle.build_csr(src, dst, w, V, np.array([0, V], np.uint32))
    with _graph(eg_lib) as g:
        g.set_option(eg.EG_OPT_SSSP_DELTA, delta)
        g.load_directed(eg.pack_edges(src, dst, w), V)
        for root in [int(src[0]), int(src[7])]:
            ref = oracle.sssp(csr["off"][0], csr["adj"], csr["w"], V, root)
            d = g.sssp(root)
            assert np.array_equal(d.view(np.uint32), ref.view(np.uint32))


def test_generator_matches_host(eg_lib):
    import torch
    import endgraph_gb300 as eg
    V, E = 100_003, 1 << 16
    for weights in [None, (0.5, 1.5)]:
        out = torch.empty((E, 3 if weights else 2), dtype=torch.int32, device="cuda")
        eg.generate_rmat(out, V, E, 99, weights=weights)
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        src, dst, w = oracle.rmat(V, E, 99, weights=weights)
        assert np.array_equal(got[:, 0], src) and np.array_equal(got[:, 1], dst)
        if weights:
            assert np.array_equal(got[:, 2], w.view(np.uint32))


def test_cpbt_kats(eg_lib):
    import endgraph_gb300 as eg
    a = [5, 0, 0, 7, 1, 0, 9, 3, 0, 2]
    assert list(eg.optimal_offset(a, 2)) == [0, 6, 10]
    assert list(eg.optimal_offset(a, 4)) == [0, 3, 6, 7, 10]
    assert list(eg.optimal_offset(a, 5)) == [0, 3, 6, 7, 10, 10]
    assert list(eg.optimal_offset([0, 0, 0, 0], 3)) == [0, 4, 4, 4]
    rng = np.random.default_rng(5)
    for n in [1, 2, 17, 1000, 30000]:
        for k in [1, 2, 3, 7, 64]:
            w = rng.integers(0, 1 << 40, n, dtype=np.uint64) * (rng.random(n) < 0.8)
            assert np.array_equal(eg.optimal_offset(w, k), oracle.optimal_offset(w, k)), (n, k)
