"""The one-partition build as one persistent cooperative launch (EG_OPT_BUILD_LAUNCH = 1, the
default) gives the same degrees, CPBT boundaries, CSR, CSC, outgoing bitmap and compressed incoming
index as the build with one launch per pass (EG_OPT_BUILD_LAUNCH = 0) and as the oracle, for one
graph and for a batch of graphs (whose ids move to the union inside the launch); the traversals
that follow see a complete graph; ids out of range are refused and leave the handle usable."""
import numpy as np
import pytest

import oracle
from helpers import graph_batch, lists_equal, rel_l1, rmat_graph

pytestmark = pytest.mark.gpu


def _structure(g):
    return dict(deg=g.degrees(), part=g.partition(), csr=g.csr(), csc=g.csc(), n=g.info().ncompressed)


def _assert_same(a, b):
    for x, y in zip(a["deg"], b["deg"]):
        assert np.array_equal(x, y)
    for x, y in zip(a["part"], b["part"]):
        assert np.array_equal(x, y)
    assert a["n"] == b["n"]
    for k in ("csr", "csc"):
        p, q = a[k], b[k]
        assert lists_equal(p["off"][0], p["adj"], q["off"][0], q["adj"], p["w"], q["w"]), k
    assert np.array_equal(a["csr"]["bitmap"], b["csr"]["bitmap"])
    assert np.array_equal(a["csc"]["cvert"], b["csc"]["cvert"])
    assert np.array_equal(a["csc"]["cidx"], b["csc"]["cidx"])


def _assert_oracle(s, src, dst, w, V):
    o_out, o_in = oracle.degrees(src, dst, V)
    assert np.array_equal(s["deg"][0], o_out) and np.array_equal(s["deg"][1], o_in)
    opo, olo = oracle.cpbt(o_out, V, 1, 1, 1, 0, True)
    assert np.array_equal(s["part"][0], opo) and np.array_equal(s["part"][1], olo)
    ref_csr = oracle.build_csr(src, dst, w, V, opo)
    ref_csc = oracle.build_csc(src, dst, w, V, opo)
    csr, csc = s["csr"], s["csc"]
    assert lists_equal(csr["off"][0], csr["adj"], ref_csr["off"][0], ref_csr["adj"], csr["w"], ref_csr["w"])
    assert lists_equal(csc["off"][0], csc["adj"], ref_csc["off"][0], ref_csc["adj"], csc["w"], ref_csc["w"])
    assert np.array_equal(csr["bitmap"], ref_csr["bitmap"])
    assert np.array_equal(csc["cvert"], ref_csc["cvert"]) and np.array_equal(csc["cidx"], ref_csc["cidx"])


@pytest.mark.parametrize("weighted", [False, True])
def test_one_launch_build_single_graph(eg_lib, weighted):
    import endgraph_gb300 as eg
    V, E = 100_000, 1_500_000
    src, dst, w = rmat_graph(V, E, 31, weights=(0.0, 1.0) if weighted else None)
    recs = eg.pack_edges(src, dst, w)
    with eg.Graph() as g:
        g.set_option(eg.EG_OPT_BUILD_LAUNCH, 0)
        g.load_directed(recs, V)
        per_pass = _structure(g)
        g.set_option(eg.EG_OPT_BUILD_LAUNCH, 1)
        g.load_directed(recs, V)
        one = _structure(g)
        pr = g.pagerank(20, 0.85)
        root = int(src[0])
        lv, _ = g.bfs(root)
        lv2, _ = g.bfs(root)  # a second traversal on the same build
    _assert_same(per_pass, one)
    _assert_oracle(one, src, dst, w, V)
    o_out, _ = oracle.degrees(src, dst, V)
    csc = oracle.build_csc(src, dst, None, V, np.array([0, V], np.uint32))
    assert rel_l1(pr, oracle.pagerank(csc["off"][0], csc["adj"], o_out, V, 20, 0.85)) <= 1e-6
    csr = oracle.build_csr(src, dst, None, V, np.array([0, V], np.uint32))
    ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, root)
    assert np.array_equal(lv, ref) and np.array_equal(lv2, ref)


@pytest.mark.parametrize("weighted", [False, True])
def test_one_launch_build_graph_batch(eg_lib, weighted):
    import endgraph_gb300 as eg
    G = 40
    Vs, eoff, parts, src, dst, w = graph_batch(G, 9, weighted)
    recs = eg.pack_edges(src, dst, w)
    rng = np.random.default_rng(4)
    roots = np.concatenate([rng.integers(0, Vs[i], 64) for i in range(G)]).astype(np.uint32)
    with eg.Graph() as g:
        g.set_option(eg.EG_OPT_BUILD_LAUNCH, 0)
        g.load_graph_batch(recs, eoff, Vs)
        per_pass = _structure(g)
        g.set_option(eg.EG_OPT_BUILD_LAUNCH, 1)
        g.load_graph_batch(recs, eoff, Vs)
        one = _structure(g)
        voff, eo = g.graph_batch()
        levels, _ = g.msbfs_graphs(roots, 64)
    assert np.array_equal(eo, eoff) and voff[-1] == Vs.sum()
    _assert_same(per_pass, one)
    # the union graph: every graph's ids shifted by its vertex offset
    gid = np.repeat(np.arange(G), np.diff(eoff.astype(np.int64)))
    base = voff[:-1].astype(np.uint64)[gid]
    us = (src.astype(np.uint64) + base).astype(np.uint32)
    ud = (dst.astype(np.uint64) + base).astype(np.uint32)
    _assert_oracle(one, us, ud, w, int(Vs.sum()))
    for i in (0, G // 2, G - 1):
        s, d, _ = parts[i]
        V = int(Vs[i])
        csr = oracle.build_csr(s, d, None, V, np.array([0, V], np.uint32))
        for j in (0, 63):
            ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, int(roots[i * 64 + j]))
            got = levels[voff[i]:voff[i + 1], j]
            assert np.array_equal(got, np.where(ref == oracle.UNREACHED, 255, ref).astype(np.uint8)), (i, j)


def test_one_launch_build_refuses_bad_ids(eg_lib):
    """A record whose id is not below its graph's vertex count stops the one-launch build with
    EndGraphError; the handle then loads and builds a valid batch as usual."""
    import endgraph_gb300 as eg
    G = 12
    Vs, eoff, _, src, dst, _ = graph_batch(G, 10)
    bad = dst.copy()
    bad[int(eoff[5]) + 3] = Vs[5]  # one past graph 5's last vertex
    with eg.Graph() as g:
        g.set_option(eg.EG_OPT_BUILD_LAUNCH, 1)
        with pytest.raises(eg.EndGraphError):
            g.load_graph_batch(eg.pack_edges(src, bad), eoff, Vs)
        g.load_graph_batch(eg.pack_edges(src, dst), eoff, Vs)
        voff, _ = g.graph_batch()
        out, _ = g.degrees()
    gid = np.repeat(np.arange(G), np.diff(eoff.astype(np.int64)))
    us = (src.astype(np.uint64) + voff[:-1].astype(np.uint64)[gid]).astype(np.uint32)
    assert np.array_equal(out, np.bincount(us, minlength=int(Vs.sum())).astype(np.uint32))


def test_one_launch_build_batch_with_edgeless_graphs(eg_lib):
    """Graphs without edges (repeated record offsets, one-vertex graphs) inside a batch: the move of
    ids to the union skips them, and the one-launch build equals the per-pass build and the oracle."""
    import endgraph_gb300 as eg
    Vs = np.array([1, 500, 1, 1, 3000, 7, 2000, 1], np.uint32)
    Es = np.array([0, 4000, 0, 0, 20000, 0, 9000, 0], np.uint64)
    parts = [rmat_graph(int(v), int(e), 300 + i) if e else (np.zeros(0, np.uint32), np.zeros(0, np.uint32), None)
             for i, (v, e) in enumerate(zip(Vs, Es))]
    eoff = np.zeros(len(Vs) + 1, np.uint64)
    eoff[1:] = np.cumsum(Es)
    src = np.concatenate([p[0] for p in parts]).astype(np.uint32)
    dst = np.concatenate([p[1] for p in parts]).astype(np.uint32)
    recs = eg.pack_edges(src, dst)
    with eg.Graph() as g:
        g.set_option(eg.EG_OPT_BUILD_LAUNCH, 0)
        g.load_graph_batch(recs, eoff, Vs)
        per_pass = _structure(g)
        g.set_option(eg.EG_OPT_BUILD_LAUNCH, 1)
        g.load_graph_batch(recs, eoff, Vs)
        one = _structure(g)
        voff, _ = g.graph_batch()
    _assert_same(per_pass, one)
    gid = np.repeat(np.arange(len(Vs)), Es.astype(np.int64))
    base = voff[:-1].astype(np.uint64)[gid]
    _assert_oracle(one, (src.astype(np.uint64) + base).astype(np.uint32),
                   (dst.astype(np.uint64) + base).astype(np.uint32), None, int(Vs.sum()))
