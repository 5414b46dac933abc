"""Edge cases through the C ABI against the oracle: empty and one-vertex graphs, self loops and
duplicate edges, a hub whose in-list is long enough for the segmented dense BFS step, a path deeper
than the captured MS-BFS loop, ids out of range, the pipelined upload of large host edge lists, and
more partitions than CPBT pages."""
import numpy as np
import pytest

import oracle
from helpers import lists_equal, rel_l1, rmat_graph

pytestmark = pytest.mark.gpu


def _ref_levels(src, dst, V, root):
    csr = oracle.build_csr(np.asarray(src, np.uint32), np.asarray(dst, np.uint32), None, V,
                           np.array([0, V], np.uint32))
    return csr, oracle.bfs_levels(csr["off"][0], csr["adj"], V, root)


def test_empty_edge_list(eg_lib):
    import endgraph_gb300 as eg
    V = 5000
    with eg.Graph() as g:
        g.load_directed(np.zeros((0, 2), np.uint32), V)
        assert g.info().E == 0
        po, _ = g.partition()
        assert po[0] == 0 and po[-1] == V
        pr = g.pagerank(20, 0.85)
        assert np.allclose(pr, 0.15)  # no in-edges: next = 1 - d every iteration
        lv, par = g.bfs(7)
        assert lv[7] == 0 and par[7] == 7
        assert np.count_nonzero(lv != oracle.UNREACHED) == 1
        levels, edges = g.msbfs(np.array([1, 2, 3], np.uint32))
        assert edges == 0 and levels[0, 1] == 0 and np.count_nonzero(levels != 255) == 3


def test_single_vertex_self_loop_and_duplicates(eg_lib):
    import endgraph_gb300 as eg
    src = np.array([0, 0, 0], np.uint32)
    dst = np.array([0, 0, 0], np.uint32)
    with eg.Graph() as g:
        g.load_directed(eg.pack_edges(src, dst), 1)
        csr, csc = g.csr(), g.csc()
        ref = oracle.build_csr(src, dst, None, 1, np.array([0, 1], np.uint32))
        assert lists_equal(csr["off"][0], csr["adj"], ref["off"][0], ref["adj"])
        assert list(csc["cvert"][:1]) == [0]
        lv, _ = g.bfs(0)
        assert list(lv) == [0]
        o_out, _ = oracle.degrees(src, dst, 1)
        refc = oracle.build_csc(src, dst, None, 1, np.array([0, 1], np.uint32))
        pr_ref = oracle.pagerank(refc["off"][0], refc["adj"], o_out, 1, 20, 0.85)
        assert rel_l1(g.pagerank(20, 0.85), pr_ref) <= 1e-6


@pytest.mark.parametrize("direction", [0, 2])
def test_hub_in_list_longer_than_a_segment(eg_lib, direction):
    """A destination with ~5000 in-edges, only one of them from the frontier and placed late in its
    list, so the dense step must walk its head and several segments before it finds a parent."""
    import endgraph_gb300 as eg
    rng = np.random.default_rng(11)
    V = 20000
    hub, root, mid = 19999, 0, 1
    feeders = rng.choice(np.arange(100, 19000), 5000, replace=False).astype(np.uint32)
    src = np.concatenate([[root], feeders, [mid], rng.integers(2, 100, 3000)]).astype(np.uint32)
    dst = np.concatenate([[mid], np.full(5000, hub), [hub], rng.integers(2, 19000, 3000)]).astype(np.uint32)
    csr, ref = _ref_levels(src, dst, V, root)
    with eg.Graph() as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        g.set_option(eg.EG_OPT_BFS_DIRECTION, direction)
        lv, par = g.bfs(root)
        assert np.array_equal(lv, ref)
        assert lv[hub] == 2 and par[hub] == mid
        assert oracle.bfs_check_parents(csr["off"][0], csr["adj"], V, root, lv, par) == 0
        levels, _ = g.msbfs(np.array([root, mid], np.uint32))
        assert np.array_equal(levels[0], np.where(ref == oracle.UNREACHED, 255, ref).astype(np.uint8))


def test_deep_path(eg_lib):
    """A 200-vertex chain: deeper than the 16 captured levels; 254 levels are the u8 limit of MS-BFS."""
    import endgraph_gb300 as eg
    n = 200
    src = np.arange(n - 1, dtype=np.uint32)
    dst = src + 1
    with eg.Graph() as g:
        g.load_directed(eg.pack_edges(src, dst), n)
        lv, _ = g.bfs(0)
        assert np.array_equal(lv, np.arange(n))
        for cg, pers in ((0, 0), (1, 0), (0, 1)):
            g.set_option(eg.EG_OPT_CUDA_GRAPH, cg)
            g.set_option(eg.EG_OPT_BATCH_LAUNCH, pers)
            levels, edges = g.msbfs(np.array([0, 50], np.uint32))
            assert np.array_equal(levels[0], np.arange(n, dtype=np.uint8))
            assert np.array_equal(levels[1][50:], np.arange(n - 50, dtype=np.uint8))
            assert np.all(levels[1][:50] == 255)
            assert edges == (n - 1) + (n - 51)
    m = 300
    src = np.arange(m - 1, dtype=np.uint32)
    with eg.Graph() as g:
        g.load_directed(eg.pack_edges(src, src + 1), m)
        with pytest.raises(eg.EndGraphError):
            g.msbfs(np.array([0], np.uint32))
        g.set_option(eg.EG_OPT_BATCH_LAUNCH, 1)
        with pytest.raises(eg.EndGraphError):
            g.msbfs(np.array([0], np.uint32))


def test_ids_out_of_range_are_rejected(eg_lib):
    import endgraph_gb300 as eg
    with eg.Graph() as g:
        with pytest.raises(eg.EndGraphError):
            g.load_directed(eg.pack_edges(np.array([0, 5], np.uint32), np.array([1, 2], np.uint32)), 5)
        # the handle stays usable after the rejected load
        g.load_directed(eg.pack_edges(np.array([0, 4], np.uint32), np.array([1, 2], np.uint32)), 5)
        lv, _ = g.bfs(0)
        assert list(lv[:2]) == [0, 1]


@pytest.mark.parametrize("weighted,pinned", [(False, False), (True, False), (False, True)])
def test_pipelined_host_load_matches_device_load(eg_lib, weighted, pinned):
    """eg_load_directed of host records with >= 2^22 edges uploads in parts and builds each part
    as it lands (ids validated in the first pass), from pinned memory directly or from pageable
    memory through the staging buffers: the same degrees, CSR, CSC, compressed index and PageRank
    as loading the records first and building after, for a ragged last part; an id >= V in the
    last part is rejected and the handle stays usable."""
    import torch

    import endgraph_gb300 as eg
    V, E = 1 << 18, (1 << 22) + 12_345
    src, dst, w = rmat_graph(V, E, 123, weights=(0.0, 1.0) if weighted else None)
    rec = eg.pack_edges(src, dst, w)
    if pinned:
        host = torch.empty(rec.shape, dtype=torch.int32, pin_memory=True)
        host.numpy()[:] = rec.view(np.int32)
        rec = host.numpy().view(np.uint32)
    with eg.Graph() as a, eg.Graph() as b:
        a.load_directed(rec, V)  # host records: pipelined upload + build
        dev = torch.from_numpy(rec.view(np.int32)).cuda()
        b.load_edges(dev, V)  # device records, loaded then built
        b.build()
        assert np.array_equal(a.degrees()[0], b.degrees()[0]) and np.array_equal(a.degrees()[1], b.degrees()[1])
        ca, cb = a.csr(), b.csr()
        assert lists_equal(ca["off"][0], ca["adj"], cb["off"][0], cb["adj"], ca["w"], cb["w"])
        assert np.array_equal(ca["bitmap"], cb["bitmap"])
        ka, kb = a.csc(), b.csc()
        assert lists_equal(ka["off"][0], ka["adj"], kb["off"][0], kb["adj"], ka["w"], kb["w"])
        assert np.array_equal(ka["cvert"], kb["cvert"]) and np.array_equal(ka["cidx"], kb["cidx"])
        o_out, _ = oracle.degrees(src, dst, V)
        assert np.array_equal(a.degrees()[0], o_out)
        assert rel_l1(a.pagerank(20, 0.85), b.pagerank(20, 0.85)) <= 1e-6
        bad = rec.copy()
        bad[E - 3, 1] = V  # a destination id out of range in the last part
        with pytest.raises(eg.EndGraphError):
            a.load_directed(bad, V)
        a.load_directed(rec, V)
        assert np.array_equal(a.degrees()[1], b.degrees()[1])
        if not weighted and not pinned:  # device memory handed over as EG_HOST: copied as such
            import ctypes
            torch.cuda.synchronize()
            st = eg_lib.eg_load_directed(a.h, ctypes.c_void_p(dev.data_ptr()), ctypes.c_uint64(E), V, 8, eg.EG_HOST)
            assert st == 0, eg_lib.eg_last_error()
            assert np.array_equal(a.degrees()[0], b.degrees()[0])


def test_pipelined_host_load_with_partitions(eg_lib):
    """P = 4 takes the generic build: the pipelined upload waits for every part, validates, and
    builds the same partitions and per-partition CSR / CSC as the device-resident load."""
    import torch

    import endgraph_gb300 as eg
    V, E = 1 << 17, (1 << 22) + 77
    src, dst, _ = rmat_graph(V, E, 321)
    rec = eg.pack_edges(src, dst)
    with eg.Graph(partitions=4) as a, eg.Graph(partitions=4) as b:
        a.load_directed(rec, V)
        b.load_edges(torch.from_numpy(rec.view(np.int32)).cuda(), V)
        b.build()
        pa, la = a.partition()
        pb, lb = b.partition()
        assert np.array_equal(pa, pb) and np.array_equal(la, lb)
        ca, cb = a.csr(), b.csr()
        ka, kb = a.csc(), b.csc()
        for p in range(4):
            assert lists_equal(ca["off"][p], ca["adj"], cb["off"][p], cb["adj"])
            assert lists_equal(ka["off"][p], ka["adj"], kb["off"][p], kb["adj"])
        bad = rec.copy()
        bad[5, 0] = V + 3
        with pytest.raises(eg.EndGraphError):
            a.load_directed(bad, V)


def test_more_partitions_than_pages(eg_lib):
    """P = 8 on a 5,000-vertex graph (two CPBT pages): most partitions are empty, as in the reference."""
    import endgraph_gb300 as eg
    rng = np.random.default_rng(2)
    V, E = 5000, 40000
    src = rng.integers(0, V, E).astype(np.uint32)
    dst = rng.integers(0, V, E).astype(np.uint32)
    o_out, _ = oracle.degrees(src, dst, V)
    ref_po, _ = oracle.cpbt(o_out, V, 8, 1, 1, 20, True)
    with eg.Graph(partitions=8) as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        po, _ = g.partition()
        assert np.array_equal(po, ref_po)
        csr, ref = _ref_levels(src, dst, V, int(src[0]))
        lv, _ = g.bfs(int(src[0]))
        assert np.array_equal(lv, ref)
        refc = oracle.build_csc(src, dst, None, V, np.array([0, V], np.uint32))
        pr_ref = oracle.pagerank(refc["off"][0], refc["adj"], o_out, V, 20, 0.85)
        assert rel_l1(g.pagerank(20, 0.85), pr_ref) <= 1e-6


def test_bounded_wait_runs_out_and_handle_survives(eg_lib):
    """A look-back wait on a descriptor that nothing publishes gives up after its poll limit: the
    call returns EG_ERR_TIMEOUT (no trap, no hang) and the same handle keeps working."""
    import endgraph_gb300 as eg
    src = np.array([0, 1, 2], np.uint32)
    dst = np.array([1, 2, 3], np.uint32)
    with eg.Graph() as g:
        assert g.selftest_bounded_wait(0) == 1  # EG_ERR_INVALID: the poll limit must be >= 1
        assert g.selftest_bounded_wait(1000) == 5  # EG_ERR_TIMEOUT
        assert b"bounded device wait" in eg_lib.eg_last_error()
        g.load_directed(eg.pack_edges(src, dst), 4)
        lv, _ = g.bfs(0)
        assert list(lv) == [0, 1, 2, 3]


def test_grid_barrier_runs_out_and_handle_survives(eg_lib):
    """The bounded grid barrier of the persistent launches: with one CTA that never arrives, the
    others give up after their poll limit, the call returns EG_ERR_TIMEOUT (no trap, no hang), and
    the same handle then builds in one persistent launch and traverses."""
    import endgraph_gb300 as eg
    src = np.array([0, 1, 2], np.uint32)
    dst = np.array([1, 2, 3], np.uint32)
    with eg.Graph() as g:
        assert g.selftest_grid_barrier(0) == 1  # EG_ERR_INVALID: the poll limit must be >= 1
        assert g.selftest_grid_barrier(1000) == 5  # EG_ERR_TIMEOUT
        assert b"bounded device wait" in eg_lib.eg_last_error()
        g.set_option(eg.EG_OPT_BUILD_LAUNCH, 1)
        g.load_directed(eg.pack_edges(src, dst), 4)
        lv, _ = g.bfs(0)
        assert list(lv) == [0, 1, 2, 3]


def test_file_ingest_matches_memory_load(eg_lib, tmp_path):
    """eg_load_file (pieces read into pinned buffers while the previous piece is copied) and
    eg_load_directed_file (read, uploaded and built in parts) load the same graph as the records
    from memory; sizes that are not a multiple of the record size, missing files and ids >= V are
    rejected."""
    import endgraph_gb300 as eg
    rng = np.random.default_rng(21)
    V, E = 50_000, 9_000_000  # 72 MB of 8-byte records: two staging pieces
    src = rng.integers(0, V, E).astype(np.uint32)
    dst = rng.integers(0, V, E).astype(np.uint32)
    w = rng.random(E).astype(np.float32)
    for weighted in (False, True):
        rec = eg.pack_edges(src, dst, w if weighted else None)
        f = tmp_path / f"g{int(weighted)}.bin"
        rec.tofile(f)
        with eg.Graph() as a, eg.Graph() as b, eg.Graph() as c:
            a.load_file(str(f), V, rec.shape[1] * 4)
            a.build()
            b.load_directed(rec, V)
            c.load_directed_file(str(f), V, rec.shape[1] * 4)  # 9 M records: four parts
            ca, cb, cc = a.csr(), b.csr(), c.csr()
            assert lists_equal(ca["off"][0], ca["adj"], cb["off"][0], cb["adj"], ca["w"], cb["w"])
            assert lists_equal(cc["off"][0], cc["adj"], cb["off"][0], cb["adj"], cc["w"], cb["w"])
            ka, kc = a.csc(), c.csc()
            assert lists_equal(kc["off"][0], kc["adj"], ka["off"][0], ka["adj"], kc["w"], ka["w"])
            assert np.array_equal(kc["cvert"], ka["cvert"]) and np.array_equal(kc["cidx"], ka["cidx"])
            assert np.array_equal(a.partition()[0], b.partition()[0])
            assert np.array_equal(c.partition()[0], b.partition()[0])
    small = tmp_path / "small.bin"  # below the pipelined size: read, then built
    eg.pack_edges(src[:1000], dst[:1000]).tofile(small)
    with eg.Graph() as g:
        g.load_directed_file(str(small), V)
        assert g.info().E == 1000 and g.info().built_csr
    oob = tmp_path / "oob.bin"
    r = eg.pack_edges(src, dst)
    r[E - 2, 1] = V
    r.tofile(oob)
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"\0" * 20)
    with eg.Graph() as g:
        with pytest.raises(eg.EndGraphError):
            g.load_file(str(bad), 10, 8)
        with pytest.raises(eg.EndGraphError):
            g.load_file(str(tmp_path / "missing.bin"), 10, 8)
        with pytest.raises(eg.EndGraphError):
            g.load_directed_file(str(bad), 10, 8)
        with pytest.raises(eg.EndGraphError):
            g.load_directed_file(str(oob), V)
        g.load_directed_file(str(small), V)  # the handle stays usable
        assert g.info().E == 1000
