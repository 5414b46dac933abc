"""CPU tests: the oracle restatement against golden vectors produced by the reference's own engine,
and (where oracle/_ref is built) against the reference directly on further seeded graphs."""
import glob
import os

import numpy as np
import pytest

import oracle
from helpers import lists_equal

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_optimal_offset_known_answers(oracle_mod):
    g = _load("optimal_offset.npz")
    a = g["kat_a"]
    for k in (1, 2, 3, 4, 5, 10, 11):
        assert np.array_equal(oracle.optimal_offset(a, k), g[f"kat_a_k{k}"]), k
    # cases checked by hand: greedy-furthest hops, zero pages join the left chunk
    assert list(g["kat_a_k2"]) == [0, 6, 10]
    assert list(g["kat_a_k4"]) == [0, 3, 6, 7, 10]
    assert list(g["kat_a_k5"]) == [0, 3, 6, 7, 10, 10]
    assert list(g["kat_zero_k3"]) == [0, 4, 4, 4]
    assert np.array_equal(oracle.optimal_offset(np.zeros(4, np.uint64), 3), g["kat_zero_k3"])
    for k in (1, 2, 7, 64):
        assert np.array_equal(oracle.optimal_offset(g["kat_rand"], k), g[f"kat_rand_k{k}"]), k


def test_cpbt_many_pages(oracle_mod):
    g = _load("cpbt_v200000_e1000000.npz")
    V, E, seed = int(g["V"]), int(g["E"]), int(g["seed"])
    src, dst, _ = oracle.rmat(V, E, seed)
    outd, ind = oracle.degrees(src, dst, V)
    n = 0
    for key in g.files:
        if not key.startswith("part_"):
            continue
        tag = key[len("part_"):]
        P, S, mode, eta = tag.split("_")
        P, S, eta = int(P[1:]), int(S[1:]), int(eta[3:])
        dense = mode == "dense"
        po, lo = oracle.cpbt(outd if dense else ind, V, P, S, eta, 20, dense)
        assert np.array_equal(po, g[key]), tag
        assert np.array_equal(lo, g[f"local_{tag}"]), tag
        n += 1
    assert n == 7 * 2 * 2 * 2


@pytest.mark.parametrize("name", ["rmat_v4096_e16384.npz", "rmat_v9000_e40000.npz", "rmat_w_v5000_e20000.npz"])
def test_structures_and_toolkits_golden(oracle_mod, name):
    g = _load(name)
    V = int(g["V"])
    src, dst = g["src"], g["dst"]
    w = g["w"] if "w" in g.files else None
    # the stored edges are the generator's
    s2, d2, w2 = oracle.rmat(V, len(src), int(g["seed"]), weights=(0.0, 1.0) if w is not None else None)
    assert np.array_equal(s2, src) and np.array_equal(d2, dst)
    outd, ind = oracle.degrees(src, dst, V)
    assert np.array_equal(outd, g["degree_out"])
    for key in g.files:
        if key.startswith("cpbt_P"):
            _, P, mode, eta = key.split("_")
            P, eta = int(P[1:]), int(eta[3:])
            dense = mode == "dense"
            po, lo = oracle.cpbt(outd if dense else ind, V, P, 2, eta, 20, dense)
            assert np.array_equal(po, g[key]), key
            assert np.array_equal(lo, g[key.replace("cpbt_", "cpbt_local_")]), key
    poff = np.array([0, V], np.uint32)
    csr = oracle.build_csr(src, dst, w, V, poff)
    csc = oracle.build_csc(src, dst, w, V, poff)
    assert lists_equal(csr["off"][0], csr["adj"], g["csr_off"], g["csr_adj"], csr["w"],
                       g["csr_w"] if w is not None else None)
    assert lists_equal(csc["off"][0], csc["adj"], g["csc_off"], g["csc_adj"], csc["w"],
                       g["csc_w"] if w is not None else None)
    assert np.array_equal(csc["cvert"], g["cvert"]) and np.array_equal(csc["cidx"], g["cidx"])
    roots = g["roots"]
    if w is None:
        pr = oracle.pagerank(csc["off"][0], csc["adj"], outd, V, 20, 0.85)
        assert np.array_equal(pr, g["pagerank20"])  # same summation order: bit-identical doubles
        for i, r in enumerate(roots):
            lv = oracle.bfs_levels(csr["off"][0], csr["adj"], V, int(r))
            assert np.array_equal(lv, g[f"bfs_level_{i}"])
            assert oracle.bfs_check_parents(csr["off"][0], csr["adj"], V, int(r), lv, g[f"bfs_parent_{i}"]) == 0
        assert np.array_equal(oracle.cc_labels(src, dst, V), g["cc_label"])
    else:
        for i, r in enumerate(roots):
            d = oracle.sssp(csr["off"][0], csr["adj"], csr["w"], V, int(r))
            assert np.array_equal(d.view(np.uint32), g[f"sssp_{i}"].view(np.uint32))


def test_bfs_parent_checker_rejects_bad_trees(oracle_mod):
    """A planted mistake in a parent array is caught (the mistake is planted on the CPU)."""
    g = _load("rmat_v4096_e16384.npz")
    V = int(g["V"])
    lv, par = g["bfs_level_0"], g["bfs_parent_0"].copy()
    csr = oracle.build_csr(g["src"], g["dst"], None, V, np.array([0, V], np.uint32))
    r = int(g["roots"][0])
    reached = np.nonzero((lv != oracle.UNREACHED) & (lv > 1))[0]
    par[reached[0]] = r  # root is not adjacent to a level >= 2 vertex at the right depth
    assert oracle.bfs_check_parents(csr["off"][0], csr["adj"], V, r, lv, par) >= 1


needs_ref = pytest.mark.skipif(not (oracle.Reference.available() or oracle.reference_dir()),
                               reason="reference engine not built here (set EG_REFERENCE_DIR to build it)")


@needs_ref
@pytest.mark.parametrize("V,E,seed", [(3000, 20000, 31), (1 << 15, 1 << 18, 32)])
def test_oracle_matches_reference_engine(oracle_mod, V, E, seed):
    if not oracle.Reference.available():
        assert oracle.build_ref() is not None
    src, dst, _ = oracle.rmat(V, E, seed)
    R = oracle.Reference(src, dst, None, V)
    R.build()
    s = R.structure()
    poff = np.array([0, V], np.uint32)
    csr = oracle.build_csr(src, dst, None, V, poff)
    csc = oracle.build_csc(src, dst, None, V, poff)
    # identical list order, not only identical lists (stable sorts, push before pull)
    assert np.array_equal(s["csr_dst"], csr["adj"])
    assert np.array_equal(s["csc_src"], csc["adj"])
    assert np.array_equal(s["cvert"], csc["cvert"]) and np.array_equal(s["cidx"], csc["cidx"])
    assert np.array_equal(s["csr_bitmap"], csr["bitmap"][0])
    outd, _ = oracle.degrees(src, dst, V)
    pr, _ = R.pagerank(20)
    assert np.array_equal(pr, oracle.pagerank(csc["off"][0], csc["adj"], outd, V, 20, 0.85))
    R.close()


def test_generator_properties(oracle_mod):
    V, E = 1 << 12, 1 << 16
    s, d, w = oracle.rmat(V, E, 5, weights=(0.5, 1.5))
    assert s.max() < V and d.max() < V
    assert w.min() >= 0.5 and w.max() < 1.5
    # edge i of a stream does not depend on where the stream is cut
    s2, d2, _ = oracle.rmat(V, 100, 5, e0=1000)
    assert np.array_equal(s2, s[1000:1100]) and np.array_equal(d2, d[1000:1100])
    # permuted ids: the R-MAT hub (id 0 before relabelling) moves
    s3, _, _ = oracle.rmat(V, E, 5, permute=False)
    assert np.bincount(s3, minlength=V).argmax() == 0
    assert np.bincount(s, minlength=V).argmax() != 0 or V == 1


def test_bc_oracle_matches_networkx(oracle_mod):
    """The reference has no BC code to pin against, so the oracle's single-source Brandes sweep is
    checked against an independent implementation: networkx's subset betweenness from one source
    (dependencies delta) and its shortest-path enumeration (path counts sigma), on a simple digraph."""
    nx = pytest.importorskip("networkx")
    rng = np.random.default_rng(5)
    V = 300
    src = rng.integers(0, V, 1500)
    dst = rng.integers(0, V, 1500)
    pairs = sorted(set((int(a), int(b)) for a, b in zip(src, dst) if a != b))
    s = np.array([p[0] for p in pairs], np.uint32)
    d = np.array([p[1] for p in pairs], np.uint32)
    csr = oracle.build_csr(s, d, None, V, np.array([0, V], np.uint32))
    G = nx.DiGraph()
    G.add_nodes_from(range(V))
    G.add_edges_from(pairs)
    for root in (0, 7, 123):
        sigma, delta, level = oracle.bc(csr["off"][0], csr["adj"], V, root)
        b = nx.betweenness_centrality_subset(G, sources=[root], targets=list(G.nodes), normalized=False)
        ref = np.array([b[v] for v in range(V)])
        mask = np.arange(V) != root
        assert np.allclose(delta[mask], ref[mask], rtol=1e-12, atol=1e-12)
        dist = nx.single_source_shortest_path_length(G, root)
        for v, lv in list(dist.items())[:25]:
            assert level[v] == lv
            if v != root:
                assert sigma[v] == sum(1 for _ in nx.all_shortest_paths(G, root, v))
