"""Batched operators through the C ABI: 64-root bit-parallel BFS and 64-source SSSP against the
oracle's single-source runs (bit-exact), personalised PageRank against an FP64 reference, and its
adjoint against FP64 autograd (dense) and FP64 central finite differences."""
import numpy as np
import pytest

import oracle
from helpers import graph_batch, rel_l1, rmat_graph

pytestmark = pytest.mark.gpu


def test_msbfs_matches_single_source(eg_lib):
    import endgraph_gb300 as eg
    V, E = 1 << 14, 1 << 18
    src, dst, _ = rmat_graph(V, E, 91)
    csr = oracle.build_csr(src, dst, None, V, np.array([0, V], np.uint32))
    rng = np.random.default_rng(3)
    roots = np.concatenate([src[rng.integers(0, E, 60)], [src[0], src[0]], rng.integers(0, V, 2)]).astype(np.uint32)
    with eg.Graph() as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        levels, edges = g.msbfs(roots)
        total = 0
        deg = np.diff(csr["off"][0].astype(np.int64))
        for s, r in enumerate(roots):
            ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, int(r))
            ref8 = np.where(ref == oracle.UNREACHED, 255, ref).astype(np.uint8)
            assert np.array_equal(levels[s], ref8), s
            total += int(deg[ref != oracle.UNREACHED].sum())
        assert edges == total


@pytest.mark.parametrize("direction_div", [20, 1, 1 << 30])  # Gemini's switch, all push, all pull
def test_msbfs_renumbered_gathers(eg_lib, direction_div):
    """Pull levels that gather through the renumbered CSC sources (and the renumbered copy of each
    frontier) give the same levels and edge count as vertex-order gathers, level by level."""
    import endgraph_gb300 as eg
    V, E = 1 << 14, 1 << 18
    src, dst, _ = rmat_graph(V, E, 93)
    csr = oracle.build_csr(src, dst, None, V, np.array([0, V], np.uint32))
    rng = np.random.default_rng(5)
    roots = src[rng.integers(0, E, 64)].astype(np.uint32)
    with eg.Graph() as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        g.set_option(eg.EG_OPT_DENSE_DIVISOR, direction_div)
        g.set_option(eg.EG_OPT_PR_RELABEL, 0)
        plain, e_plain = g.msbfs(roots)
        g.set_option(eg.EG_OPT_PR_RELABEL, 1)
        ren, e_ren = g.msbfs(roots)
        assert np.array_equal(plain, ren) and e_plain == e_ren
        for s in (0, 17, 63):
            ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, int(roots[s]))
            assert np.array_equal(ren[s], np.where(ref == oracle.UNREACHED, 255, ref).astype(np.uint8))
        run = g.last_run()
        if direction_div == 1:
            assert run["pull"] == 0
        if direction_div == 1 << 30:
            assert run["push"] == 0


@pytest.mark.parametrize("cuda_graph,persistent", [(0, 0), (1, 0), (0, 1)])
def test_msbfs_cuda_graph_mode(eg_lib, cuda_graph, persistent):
    """The captured level loop and the persistent launch (each level choosing push or pull on the
    device) give the same levels as the host-driven loop, and take both directions as it does."""
    import endgraph_gb300 as eg
    V, E = 1 << 13, 1 << 16
    src, dst, _ = rmat_graph(V, E, 97)
    csr = oracle.build_csr(src, dst, None, V, np.array([0, V], np.uint32))
    roots = np.array(src[:64], np.uint32)
    with eg.Graph() as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        g.set_option(eg.EG_OPT_CUDA_GRAPH, cuda_graph)
        g.set_option(eg.EG_OPT_BATCH_LAUNCH, persistent)
        for rep in range(2):  # the second call replays the cached graph
            levels, _ = g.msbfs(roots[rep * 8:] if rep else roots)
            use = roots[rep * 8:] if rep else roots
            run = g.last_run()
            assert run["push"] > 0 and run["pull"] > 0  # both directions, chosen on the device when captured
            for s in (0, 5, len(use) - 1):
                ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, int(use[s]))
                assert np.array_equal(levels[s], np.where(ref == oracle.UNREACHED, 255, ref).astype(np.uint8))


def test_autotune_keeps_results(eg_lib):
    """The tuner only changes how the work is scheduled: results after tuning equal the oracle."""
    import endgraph_gb300 as eg
    V, E = 1 << 15, 1 << 19
    src, dst, _ = rmat_graph(V, E, 98)
    csr = oracle.build_csr(src, dst, None, V, np.array([0, V], np.uint32))
    roots = np.array(src[:70], np.uint32)
    with eg.Graph() as g:
        g.load_directed(eg.pack_edges(src, dst), V)
        t = g.autotune(roots[:8])
        assert t["batch_width"] in (16, 32, 64) and t["cuda_graph"] in (0, 1)
        assert t["batch_divisor"] in (5, 10, 20, 40)
        assert t["bfs_ms"] > 0 and t["pull_sweep_ms"] > 0
        lv, _ = g.bfs(int(roots[0]))
        assert np.array_equal(lv, oracle.bfs_levels(csr["off"][0], csr["adj"], V, int(roots[0])))
        levels = np.empty((70, V), np.uint8)
        g.bfs_many(roots, levels)
        for s in (0, 33, 69):
            ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, int(roots[s]))
            assert np.array_equal(levels[s], np.where(ref == oracle.UNREACHED, 255, ref).astype(np.uint8))


@pytest.mark.parametrize("cuda_graph,persistent", [(0, 0), (1, 0), (0, 1)])
def test_graph_batch_msbfs(eg_lib, cuda_graph, persistent):
    """Many small graphs preprocessed together; 64 roots per graph; every graph matches the oracle."""
    import endgraph_gb300 as eg
    G = 40
    Vs, eoff, parts, src, dst, _ = graph_batch(G, 7)
    rng = np.random.default_rng(1)
    roots = np.concatenate([rng.integers(0, Vs[i], 64) for i in range(G)]).astype(np.uint32)
    with eg.Graph() as g:
        g.load_graph_batch(eg.pack_edges(src, dst), eoff, Vs)
        g.set_option(eg.EG_OPT_CUDA_GRAPH, cuda_graph)
        g.set_option(eg.EG_OPT_BATCH_LAUNCH, persistent)
        voff, eo = g.graph_batch()
        assert np.array_equal(eo, eoff) and voff[-1] == Vs.sum()
        levels, _ = g.msbfs_graphs(roots, 64)
    for i in (0, 1, G // 2, G - 1):
        s, d, _ = parts[i]
        V = int(Vs[i])
        csr = oracle.build_csr(s, d, None, V, np.array([0, V], np.uint32))
        block = levels[voff[i]:voff[i + 1]]
        for j in (0, 17, 63):
            ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, int(roots[i * 64 + j]))
            assert np.array_equal(block[:, j], np.where(ref == oracle.UNREACHED, 255, ref).astype(np.uint8)), (i, j)


def test_graph_batch_sssp(eg_lib):
    import endgraph_gb300 as eg
    G = 24
    Vs, eoff, parts, src, dst, w = graph_batch(G, 8, weighted=True)
    rng = np.random.default_rng(2)
    sources = np.concatenate([rng.integers(0, Vs[i], 64) for i in range(G)]).astype(np.uint32)
    with eg.Graph() as g:
        g.load_graph_batch(eg.pack_edges(src, dst, w), eoff, Vs)
        voff, _ = g.graph_batch()
        dist = g.sssp_graphs(sources, 64)
    for i in (0, G // 3, G - 1):
        s, d, ww = parts[i]
        V = int(Vs[i])
        csr = oracle.build_csr(s, d, ww, V, np.array([0, V], np.uint32))
        for j in (0, 31, 63):
            ref = oracle.sssp(csr["off"][0], csr["adj"], csr["w"], V, int(sources[i * 64 + j]))
            got = dist[voff[i]:voff[i + 1], j]
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (i, j)


def test_sssp_batch_matches_single_source(eg_lib):
    import endgraph_gb300 as eg
    V, E = 1 << 13, 1 << 17
    src, dst, w = rmat_graph(V, E, 92, weights=(0.0, 1.0))
    csr = oracle.build_csr(src, dst, w, V, np.array([0, V], np.uint32))
    sources = np.array([src[0], src[9], dst[4], 7, src[100]] + list(src[200:259]), np.uint32)
    with eg.Graph() as g:
        g.load_directed(eg.pack_edges(src, dst, w), V)
        dist = g.sssp_batch(sources)
    for s, r in enumerate(sources):
        ref = oracle.sssp(csr["off"][0], csr["adj"], csr["w"], V, int(r))
        assert np.array_equal(dist[s].view(np.uint32), ref.view(np.uint32)), s


def _ppr_fp64(src, dst, w, V, seeds, alpha, K):
    """Dense FP64 power iteration (torch, on w's device), differentiable in w."""
    import torch
    n = len(seeds)
    dev = w.device
    s_idx = torch.as_tensor(src, dtype=torch.long, device=dev)
    d_idx = torch.as_tensor(dst, dtype=torch.long, device=dev)
    s_out = torch.zeros(V, dtype=torch.float64, device=dev).index_add(0, s_idx, w)
    a_val = w / s_out[s_idx]
    e = torch.zeros(V, n, dtype=torch.float64, device=dev)
    e[torch.as_tensor(seeds, dtype=torch.long, device=dev), torch.arange(n, device=dev)] = 1.0
    A = torch.zeros(V, V, dtype=torch.float64, device=dev).index_put((s_idx, d_idx), a_val, accumulate=True)
    x = e.clone()
    for _ in range(K):
        x = alpha * e + (1 - alpha) * (A.T @ x)
    return x.T  # [n][V]


def _small_graph(V, E, seed):
    src, dst, _ = rmat_graph(V, E, seed)
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.5, 1.5, E).astype(np.float32)  # U[0.5, 1.5)
    return src, dst, w


def test_ppr_forward_fp64(eg_lib):
    import torch
    import endgraph_gb300 as eg
    V, E, K, alpha = 1024, 16384, 50, 0.15
    src, dst, w = _small_graph(V, E, 93)
    seeds = np.array(src[:64], np.uint32)
    with eg.Graph() as g:
        g.load_directed_with_ids(eg.pack_edges(src, dst), V)
        x = g.ppr(w, seeds, alpha, K)
    ref = _ppr_fp64(src, dst, torch.as_tensor(w, dtype=torch.float64), V, seeds, alpha, K).numpy()
    assert rel_l1(x, ref) <= 1e-6, rel_l1(x, ref)


def test_ppr_single_seed_path(eg_lib):
    """One seed takes the scalar pull path; it must agree with FP64 and with the 64-column engine."""
    import torch
    import endgraph_gb300 as eg
    V, E, K, alpha = 1 << 14, 1 << 18, 50, 0.15
    src, dst, w = _small_graph(V, E, 95)
    seeds = np.array(src[:8], np.uint32)
    with eg.Graph() as g:
        g.load_directed_with_ids(eg.pack_edges(src, dst), V)
        xb = g.ppr(w, seeds, alpha, K)
        for i, s in enumerate(seeds):
            x1 = g.ppr(w, np.array([s], np.uint32), alpha, K)
            assert rel_l1(x1[0], xb[i]) <= 1e-6
    ref = _ppr_fp64(src, dst, torch.as_tensor(w, dtype=torch.float64, device="cuda"), V, seeds[:2], alpha, K)
    assert rel_l1(xb[:2], ref.cpu().numpy()) <= 1e-6


class _PPR:
    """torch.autograd.Function over the C-ABI forward / backward (test harness only)."""

    @staticmethod
    def make(g, seeds, alpha, K):
        import torch

        class F(torch.autograd.Function):
            @staticmethod
            def forward(ctx, w):
                ctx.save_for_backward(w)
                out = torch.empty((len(seeds), g.info().V), dtype=torch.float32, device=w.device)
                g.ppr(w, seeds, alpha, K, out=out)
                return out

            @staticmethod
            def backward(ctx, grad_out):
                (w,) = ctx.saved_tensors
                dw = torch.empty_like(w)
                g.ppr_backward(w, seeds, grad_out.contiguous(), alpha, K, dl_dw=dw)
                return dw

        return F


def test_ppr_adjoint_against_fp64_autograd_and_finite_differences(eg_lib):
    import torch
    import endgraph_gb300 as eg
    V, E, K, alpha = 1024, 8192, 50, 0.15
    src, dst, w = _small_graph(V, E, 94)
    seeds = np.array(src[:64], np.uint32)
    rng = np.random.default_rng(5)
    target = rng.random((64, V)) * 2.0 / V
    with eg.Graph() as g:
        g.load_directed_with_ids(eg.pack_edges(src, dst), V)
        F = _PPR.make(g, seeds, alpha, K)
        wt = torch.tensor(w, device="cuda", requires_grad=True)
        x = F.apply(wt)
        loss = ((x - torch.as_tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
        loss.backward()
        grad = wt.grad.cpu().numpy().astype(np.float64)
    # dense FP64 reference gradient
    w64 = torch.tensor(w, dtype=torch.float64, requires_grad=True)
    x64 = _ppr_fp64(src, dst, w64, V, seeds, alpha, K)
    l64 = ((x64 - torch.as_tensor(target)) ** 2).sum()
    l64.backward()
    g64 = w64.grad.numpy()
    rel = np.linalg.norm(grad - g64) / np.linalg.norm(g64)
    assert rel <= 1e-4, rel
    # FP64 central finite differences on 256 random edges
    idx = rng.choice(E, 256, replace=False)
    h = 1e-6
    fd = np.empty(256)
    with torch.no_grad():
        base = torch.tensor(w, dtype=torch.float64, device="cuda")
        tgt = torch.as_tensor(target, device="cuda")
        for j, i in enumerate(idx):
            wp = base.clone()
            wp[i] += h
            wm = base.clone()
            wm[i] -= h
            lp = ((_ppr_fp64(src, dst, wp, V, seeds, alpha, K) - tgt) ** 2).sum().item()
            lm = ((_ppr_fp64(src, dst, wm, V, seeds, alpha, K) - tgt) ** 2).sum().item()
            fd[j] = (lp - lm) / (2 * h)
    err = np.linalg.norm(grad[idx] - fd) / np.linalg.norm(fd)
    assert err <= 1e-3, err
