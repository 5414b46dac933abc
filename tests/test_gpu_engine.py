"""The device operator API (include/endgraph_gb300_engine.cuh): the four reference toolkits written
as signal/slot device functors (tests/engine/engine_toolkits.cu) against the oracle.  With several
CPBT partitions every step goes through the master/mirror message path (per-partition buffers of
{vertex, message} pairs, core/graph.hpp:1445-1470, :1505-1802); the run's JSON line reports the
messages, so the tests check that they flowed."""
import json
import os
import subprocess

import numpy as np
import pytest

import oracle
from helpers import rel_l1, rmat_graph

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "engine", "engine_toolkits.cu")
LIBDIR = os.path.join(ROOT, "endgraph_gb300")


def _compile(out):
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
           "-I", os.path.join(ROOT, "include"), SRC, "-o", out, "-L", LIBDIR, "-lendgraph_gb300",
           "-Xlinker", f"-rpath={LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return out


def test_engine_header_compiles_for_sm103a(tmp_path):
    from endgraph_gb300 import build
    build.build()
    _compile(str(tmp_path / "engine_toolkits"))


@pytest.fixture(scope="module")
def engine_exe(tmp_path_factory):
    from endgraph_gb300 import build
    build.build()
    return _compile(str(tmp_path_factory.mktemp("engine") / "engine_toolkits"))


def _check_messages(log, P, selective=False):
    st = json.loads(log.strip().splitlines()[-1])
    if P > 1:
        assert st["messages"] > 0 and st["message_bytes"] > 0, st
        if selective:
            assert st["selective_bytes"] > 0, st
    else:
        assert st["messages"] == 0, st
    return st


def _run(exe, tmp_path, algo, rec, V, arg, partitions=1):
    f = tmp_path / f"{algo}.bin"
    rec.tofile(f)
    out = tmp_path / f"{algo}.out"
    r = subprocess.run([exe, algo, str(f), str(V), str(arg), str(out), str(partitions)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return out, r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("V,E,seed,P", [(1 << 14, 1 << 18, 5, 1), (100_000, 600_000, 6, 1), (100_000, 600_000, 6, 2),
                                        (100_000, 600_000, 6, 4)])
def test_engine_pagerank_fp64(engine_exe, tmp_path, V, E, seed, P):
    import endgraph_gb300 as eg
    src, dst, _ = rmat_graph(V, E, seed)
    out, log = _run(engine_exe, tmp_path, "pagerank", eg.pack_edges(src, dst), V, 20, P)
    _check_messages(log, P)
    pr = np.fromfile(out, np.float64)
    o_out, _ = oracle.degrees(src, dst, V)
    csc = oracle.build_csc(src, dst, None, V, np.array([0, V], np.uint32))
    ref = oracle.pagerank(csc["off"][0], csc["adj"], o_out, V, 20, 0.85)
    assert rel_l1(pr, ref) <= 1e-12  # both FP64; only the summation order differs


@pytest.mark.gpu
@pytest.mark.parametrize("V,E,seed,P", [(1 << 14, 1 << 18, 7, 1), (1 << 16, 1 << 20, 8, 1), (1 << 16, 1 << 20, 8, 2),
                                        (1 << 16, 1 << 20, 8, 4)])
def test_engine_bfs(engine_exe, tmp_path, V, E, seed, P):
    import endgraph_gb300 as eg
    src, dst, _ = rmat_graph(V, E, seed)
    root = int(src[0])
    out, log = _run(engine_exe, tmp_path, "bfs", eg.pack_edges(src, dst), V, root, P)
    a = np.fromfile(out, np.uint32)
    lv, par = a[:V], a[V:]
    csr = oracle.build_csr(src, dst, None, V, np.array([0, V], np.uint32))
    assert np.array_equal(lv, oracle.bfs_levels(csr["off"][0], csr["adj"], V, root))
    assert oracle.bfs_check_parents(csr["off"][0], csr["adj"], V, root, lv, par) == 0
    assert '"dense_steps": 0' not in log  # the E/20 switch took the pull path at least once
    _check_messages(log, P, selective=True)  # visited is the dense_selective subset


@pytest.mark.gpu
@pytest.mark.parametrize("V,E,seed,P", [(1 << 14, 1 << 17, 9, 1), (100_000, 300_000, 10, 1), (100_000, 300_000, 10, 2),
                                        (100_000, 300_000, 10, 4)])
def test_engine_cc(engine_exe, tmp_path, V, E, seed, P):
    import endgraph_gb300 as eg
    src, dst, _ = rmat_graph(V, E, seed)
    out, log = _run(engine_exe, tmp_path, "cc", eg.pack_edges(src, dst), V, 0, P)
    _check_messages(log, P)
    assert np.array_equal(np.fromfile(out, np.uint32), oracle.cc_labels(src, dst, V))


@pytest.mark.gpu
@pytest.mark.parametrize("V,E,seed,P", [(1 << 14, 1 << 17, 11, 1), (50_000, 400_000, 12, 1), (50_000, 400_000, 12, 2),
                                        (50_000, 400_000, 12, 4)])
def test_engine_sssp(engine_exe, tmp_path, V, E, seed, P):
    import endgraph_gb300 as eg
    src, dst, w = rmat_graph(V, E, seed, weights=(0.0, 1.0))
    root = int(src[0])
    out, log = _run(engine_exe, tmp_path, "sssp", eg.pack_edges(src, dst, w), V, root, P)
    _check_messages(log, P)
    d = np.fromfile(out, np.float32)
    csr = oracle.build_csr(src, dst, w, V, np.array([0, V], np.uint32))
    ref = oracle.sssp(csr["off"][0], csr["adj"], csr["w"], V, root)
    assert np.array_equal(d.view(np.uint32), ref.view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("V,E,seed", [(1 << 12, 1 << 15, 13), (1 << 16, 1 << 20, 14)])
def test_bc_toolkit(tmp_path, V, E, seed):
    """Betweenness dependencies from the bc toolkit (forward path counting, backward sweep on the
    transposed graph through set_transposed) against Brandes' algorithm in the oracle: path counts
    bit-exact, dependencies within 1e-9 relative L1 (FP64 sums in another order)."""
    import endgraph_gb300 as eg
    from endgraph_gb300 import build
    bindir = build.build_toolkits()
    src, dst, _ = rmat_graph(V, E, seed)
    f = tmp_path / "g.bin"
    eg.pack_edges(src, dst).tofile(f)
    root = int(src[0])
    out = tmp_path / "bc.out"
    r = subprocess.run([os.path.join(bindir, "bc"), str(f), str(V), str(root), "1", str(out)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    a = np.fromfile(out, np.float64)
    sigma, delta = a[:V], a[V:]
    csr = oracle.build_csr(src, dst, None, V, np.array([0, V], np.uint32))
    rs, rd, _ = oracle.bc(csr["off"][0], csr["adj"], V, root)
    assert np.array_equal(sigma, rs)
    assert rel_l1(delta, rd) <= 1e-9
