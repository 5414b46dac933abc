"""Parity at full size: the GPU build and toolkits against the reference's own engine (oracle/_ref,
core/graph.hpp compiled at one rank) on the same seeded graphs as the benchmark.

* The bench workload: R-MAT with 2^25 vertices and 2^29 edges, ids permuted -- degrees, the CPBT
  partition, the CSR (index at every source, source bitmap, per-list neighbour signatures), the
  CSC (compressed index, per-list signatures), PageRank x20 (FP32 against the reference's FP64,
  relative L1 <= 1e-6) and BFS levels from the bench's 16 roots (bit-exact, parents a BFS tree).
* A power-law stand-in for the twitter-2010-sized configuration at 2^24 vertices and 2^29
  weighted edges: SSSP distances bit-exact, and CC labels bit-exact on the symmetrised graph
  (2^30 edges).
* The differentiable personalised PageRank at 2^22 vertices and 2^26 edges: forward and adjoint
  against FP64 (no reference counterpart: it is a growth pattern of this library).

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


def test_ppr_adjoint_at_size(eg_lib):
    """The differentiable personalised PageRank at its full size: 2^22 vertices, 2^26 edges, learnable
    weights w ~ U[0.5, 1.5) row-normalised, teleport 0.15, K = 50, loss = squared L2 distance to
    seeded random targets.  The FP32 adjoint (transposed power iteration over the CSR with
    checkpoints every ceil(sqrt(K)) steps) against FP64 central differences on 256 random edges.
    Two seeds: the differences need 1 + 2 x 256 FP64 solves per seed, run together as the columns
    of one sparse power iteration in which every perturbed column adds the change of its edge's
    row (the row is renormalised, so every out-edge of the perturbed source moves).  An FP64 adjoint
    of the same iteration (torch sparse products) checks the differences and, over every edge, the
    FP32 gradient."""
    import torch

    import endgraph_gb300 as eg
    V, E, K, alpha, h, M = 1 << 22, 1 << 26, 50, 0.15, 1e-5, 256
    dev = torch.device("cuda")
    ep = torch.empty((E, 2), dtype=torch.int32, device=dev)
    eg.generate_rmat(ep, V, E, SEED + 7, 0.57, 0.19, 0.19, permute=True)
    gen = torch.Generator(device="cpu").manual_seed(SEED)
    w = (torch.rand(E, generator=gen, dtype=torch.float32) + 0.5).to(dev)
    seeds = ep[:2, 0].cpu().numpy().view(np.uint32).copy()
    ns = len(seeds)
    tgt = (torch.rand((ns, V), generator=gen, dtype=torch.float64) * (2.0 / V)).to(dev)
    with eg.Graph(eta=1) as g:
        g.load_directed_with_ids(ep, V)
        x = torch.empty((ns, V), dtype=torch.float32, device=dev)
        g.ppr(w, seeds, alpha, K, out=x)
        dl = (2.0 * (x.double() - tgt)).float().contiguous()
        dw = torch.empty_like(w)
        g.ppr_backward(w, seeds, dl, alpha, K, dl_dw=dw)
        torch.cuda.synchronize()
    grad = dw.double()
    # FP64 operator A^T (A_uv = w_uv / sum of u's weights) as CSR
    src, dst = ep[:, 0].long(), ep[:, 1].long()
    del ep
    w64 = w.double()
    s_out = torch.zeros(V, dtype=torch.float64, device=dev).index_add_(0, src, w64)
    a = w64 / s_out[src]
    AT = torch.sparse_coo_tensor(torch.stack([dst, src]), a, (V, V)).coalesce().to_sparse_csr()
    A = torch.sparse_coo_tensor(torch.stack([src, dst]), a, (V, V)).coalesce().to_sparse_csr()
    # FP64 adjoint of the same unrolled iteration: x_k kept, lambda_K = 2 (x_K - t),
    # G_e += (1-a) x_k[u] lambda_{k+1}[v], lambda_k = (1-a) A lambda_{k+1}
    e_cols = torch.zeros((V, ns), dtype=torch.float64, device=dev)
    e_cols[torch.as_tensor(seeds.astype(np.int64), device=dev), torch.arange(ns, device=dev)] = 1.0
    xs = [e_cols]
    for _ in range(K):
        xs.append(alpha * e_cols + (1.0 - alpha) * torch.sparse.mm(AT, xs[-1]))
    lam = 2.0 * (xs[K] - tgt.T)
    G = torch.zeros(E, dtype=torch.float64, device=dev)
    for k in range(K - 1, -1, -1):
        G += (1.0 - alpha) * (xs[k][src] * lam[dst]).sum(1)
        lam = (1.0 - alpha) * torch.sparse.mm(A, lam)
    del xs, lam, A
    dot = torch.zeros(V, dtype=torch.float64, device=dev).index_add_(0, src, a * G)
    exact = (G - dot[src]) / s_out[src]
    del G, dot
    # the out-edges of each perturbed edge's source
    rng = np.random.default_rng(SEED)
    idx = torch.as_tensor(rng.choice(E, M, replace=False), device=dev)
    order = torch.argsort(src)
    offs = torch.searchsorted(src[order], torch.arange(V + 1, device=dev))
    C1 = 1 + 2 * M
    ents_v, ents_u, ents_c, ents_d = [], [], [], []
    for j in range(M):
        e = int(idx[j])
        u = int(src[e])
        row = order[int(offs[u]):int(offs[u + 1])]
        for k, sign in ((1, 1.0), (2, -1.0)):
            s2 = s_out[u] + sign * h
            wp = w64[row] + sign * h * (row == e).double()
            delta = wp / s2 - a[row]
            for s in range(ns):
                ents_v.append(dst[row])
                ents_u.append(torch.full_like(row, u))
                ents_c.append(torch.full_like(row, s * C1 + 1 + 2 * j + (k - 1)))
                ents_d.append(delta)
    ev, eu, ec, ed = (torch.cat(t) for t in (ents_v, ents_u, ents_c, ents_d))
    del src, dst, order, offs
    # FP64 power iterations of all columns: seed s owns columns [s C1, (s+1) C1): its base solution
    # x, then for every edge the change of the solution under +h and under -h.  A perturbed
    # solution is carried as its difference D from the base (D_0 = 0, D_{k+1} = (1-a) (A^T D_k +
    # dA^T (x_k + D_k))), so the differences never come out of two large, nearly equal numbers.
    C = ns * C1
    X = torch.zeros((V, C), dtype=torch.float64, device=dev)
    seeds_t = torch.as_tensor(seeds.astype(np.int64), device=dev)
    base_cols = torch.arange(ns, device=dev) * C1
    X[seeds_t, base_cols] = 1.0
    ebase = (ec // C1) * C1
    for _ in range(K):
        Y = torch.sparse.mm(AT, X)
        Y.index_put_((ev, ec), ed * (X[eu, ebase] + X[eu, ec]), accumulate=True)
        Y.mul_(1.0 - alpha)
        Y[seeds_t, base_cols] += alpha
        X = Y
        del Y
    # the forward at size: FP32 against the FP64 base columns
    base = X[:, base_cols].T
    fwd_err = float((x.double() - base).abs().sum() / base.abs().sum())
    fd = torch.zeros(M, dtype=torch.float64, device=dev)
    for s in range(ns):
        dp = X[:, s * C1 + 1:(s + 1) * C1:2]
        dm = X[:, s * C1 + 2:(s + 1) * C1:2]
        r = 2.0 * (X[:, s * C1] - tgt[s])[:, None]
        fd += ((dp - dm) * (r + dp + dm)).sum(0) / (2.0 * h)
    got = grad[idx]
    err = float(torch.linalg.norm(got - fd) / torch.linalg.norm(fd))
    harness = float(torch.linalg.norm(exact[idx] - fd) / torch.linalg.norm(fd))
    err_all = float(torch.linalg.norm(grad - exact) / torch.linalg.norm(exact))
    print(f"PPR adjoint 2^22/2^26, K={K}, {ns} seeds: forward rel L1 vs FP64 {fwd_err:.2e}; "
          f"gradient on {M} random edges rel L2 vs FP64 central differences {err:.2e} "
          f"(|fd| max {float(fd.abs().max()):.3e}); FP64 adjoint vs the differences {harness:.2e}; "
          f"all {E} edges vs the FP64 adjoint {err_all:.2e}")
    assert fwd_err <= 1e-6, fwd_err      # measured 2.2e-7
    assert harness <= 1e-5, harness      # measured 2.7e-7
    assert err <= 1e-4, err              # measured 9.0e-7
    assert err_all <= 1e-4, err_all      # measured 7.7e-7
