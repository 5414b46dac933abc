"""The C++ Graph<EdgeData> surface (include/core/graph.hpp): the reference's toolkits compile
unchanged against it, and the C++ toolkit programs built on it reproduce the oracle on the GPU."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from helpers import rel_l1

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
REF_TOOLKITS = "/root/reference/toolkits"


def _lib_dir():
    from endgraph_gb300 import build
    build.build()
    return os.path.dirname(build.LIB)


@pytest.mark.skipif(not os.path.isdir(REF_TOOLKITS), reason="reference toolkits not present on this machine")
@pytest.mark.parametrize("name", ["pagerank", "bfs", "cc", "sssp"])
def test_reference_toolkits_compile_unchanged(name, tmp_path):
    lib = _lib_dir()
    src = os.path.join(REF_TOOLKITS, f"{name}.cpp")
    exe = tmp_path / name
    r = subprocess.run(["g++", "-std=c++14", "-O1", f"-I{INCLUDE}", src, "-o", str(exe), f"-L{lib}",
                        "-lendgraph_gb300", f"-Wl,-rpath,{lib}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()


def test_cpp_toolkits_build():
    from endgraph_gb300 import build
    d = build.build_toolkits()
    for t in build.TOOLKITS:
        assert os.path.exists(os.path.join(d, t))


def _write_edges(path, src, dst, w=None):
    import endgraph_gb300 as eg
    eg.pack_edges(src, dst, w).tofile(path)


@pytest.mark.gpu
def test_cpp_toolkits_match_oracle(eg_lib):
    from endgraph_gb300 import build
    d = build.build_toolkits()
    V, E = 20_000, 200_000
    src, dst, _ = oracle.rmat(V, E, 61)
    sw, dw, w = oracle.rmat(V, E, 62, weights=(0.0, 1.0))
    poff = np.array([0, V], np.uint32)
    with tempfile.TemporaryDirectory() as tmp:
        f = os.path.join(tmp, "g.bin")
        fw = os.path.join(tmp, "gw.bin")
        _write_edges(f, src, dst)
        _write_edges(fw, sw, dw, w)
        out = os.path.join(tmp, "out.bin")

        def run(tk, graph, arg):
            r = subprocess.run([os.path.join(d, tk), graph, str(V), str(arg), "1", out], capture_output=True,
                               text=True, timeout=300)
            assert r.returncode == 0, r.stderr
            return r.stdout

        outd, _ = oracle.degrees(src, dst, V)
        csc = oracle.build_csc(src, dst, None, V, poff)
        run("pagerank", f, 20)
        pr = np.fromfile(out, np.float32)
        assert rel_l1(pr, oracle.pagerank(csc["off"][0], csc["adj"], outd, V, 20, 0.85)) <= 1e-6
        root = int(src[0])
        txt = run("bfs", f, root)
        csr = oracle.build_csr(src, dst, None, V, poff)
        lv = np.fromfile(out, np.uint32)
        ref = oracle.bfs_levels(csr["off"][0], csr["adj"], V, root)
        assert np.array_equal(lv, ref)
        assert f"found_vertices = {int((ref != oracle.UNREACHED).sum())}" in txt
        run("cc", f, 0)
        assert np.array_equal(np.fromfile(out, np.uint32), oracle.cc_labels(src, dst, V))
        rootw = int(sw[0])
        run("sssp", fw, rootw)
        csrw = oracle.build_csr(sw, dw, w, V, poff)
        ref = oracle.sssp(csrw["off"][0], csrw["adj"], csrw["w"], V, rootw)
        assert np.array_equal(np.fromfile(out, np.float32).view(np.uint32), ref.view(np.uint32))


HOST_CALLBACK_PROGRAM = r"""
#include "core/graph.hpp"
int main(int argc, char** argv) {
    Graph<Empty> g(1);
    g.load_directed(argv[1], (UINT)atoi(argv[2]));
    VertexSubset* active = g.alloc_vertex_subset();
    active->fill();
    try {
        g.process_vertices<UINT>([&](UINT v) { return v; }, active);
    } catch (const EndGraphError& e) {
        printf("refused status=%d\n", e.status);
        delete active;
        return 0;
    }
    return 3;
}
"""


@pytest.mark.gpu
def test_host_callbacks_are_refused_loudly(eg_lib, tmp_path):
    lib = _lib_dir()
    src_file = tmp_path / "hc.cpp"
    src_file.write_text(HOST_CALLBACK_PROGRAM)
    exe = tmp_path / "hc"
    r = subprocess.run(["g++", "-std=c++14", f"-I{INCLUDE}", str(src_file), "-o", str(exe), f"-L{lib}",
                        "-lendgraph_gb300", f"-Wl,-rpath,{lib}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    s, d, _ = oracle.rmat(1000, 5000, 3)
    g = tmp_path / "g.bin"
    _write_edges(str(g), s, d)
    r = subprocess.run([str(exe), str(g), "1000"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "refused status=6" in r.stdout
