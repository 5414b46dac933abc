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
_REF = oracle.reference_dir()  # $EG_REFERENCE_DIR or the checkout oracle/build_ref.sh compiled
REF_TOOLKITS = os.path.join(_REF, "toolkits") if _REF else ""


def _lib_dir():
    from endgraph_gb300 import build
    build.build()
    return os.path.dirname(build.LIB)


@pytest.mark.skipif(not REF_TOOLKITS or not os.path.isdir(REF_TOOLKITS),
                    reason="reference toolkits not present on this machine (set EG_REFERENCE_DIR)")
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


PERSIST_PROGRAM = r"""
#include "core/graph.hpp"
// Dumps the PageRank result with the header's dump_vertex_array, restores it into a second array
// and writes both to stdout as one result line; checks the reference's file rules on the way.
int main(int argc, char** argv) {
    Graph<Empty> g(1);
    g.load_directed(argv[1], (UINT)atoi(argv[2]));
    const std::string path = argv[3];
    float* pr = g.alloc_vertex_array<float>();
    g.pagerank(20, pr);
    // a stale file of another size is replaced by one of sizeof(T) * V bytes
    FILE* f = fopen(path.c_str(), "wb");
    fputs("stale", f);
    fclose(f);
    g.dump_vertex_array(pr, path);
    long size_after_dump = file_size(path);
    float* back = g.alloc_vertex_array<float>();
    g.fill_vertex_array(back, -1.0f);
    g.restore_vertex_array(back, path);
    int same = memcmp(pr, back, sizeof(float) * g.vertices_num) == 0;
    // a file of the right size is rewritten in place
    double* d = g.alloc_vertex_array<double>();
    for (UINT v = 0; v < g.vertices_num; ++v) d[v] = 0.5 * v;
    const std::string dpath = path + ".f64";
    g.dump_vertex_array(d, dpath);
    for (UINT v = 0; v < g.vertices_num; ++v) d[v] = 2.0 * v;
    g.dump_vertex_array(d, dpath);
    double* d2 = g.alloc_vertex_array<double>();
    g.restore_vertex_array(d2, dpath);
    int same_d = memcmp(d, d2, sizeof(double) * g.vertices_num) == 0;
    int refused = 0;
    try {
        UINT* wrong = g.alloc_vertex_array<UINT>();
        g.restore_vertex_array(wrong, dpath);  // 8 V bytes on disk, 4 V expected
    } catch (const EndGraphError& e) {
        refused = e.status == EG_ERR_INVALID;
    }
    g.gather_vertex_array(pr, 0);
    printf("size=%ld same=%d same_d=%d size_d=%ld refused=%d\n", size_after_dump, same, same_d, file_size(dpath),
           refused);
    return 0;
}
"""


@pytest.mark.gpu
def test_vertex_array_persistence(eg_lib, tmp_path):
    """dump_vertex_array / restore_vertex_array of the C++ header keep the reference's file format
    (core/graph.hpp:325-378): a raw sizeof(T) * V file, created at that size when missing or of
    another size, rewritten in place otherwise, and refused on restore when its size differs.  The
    dumped file holds the GPU's PageRank result byte for byte."""
    lib = _lib_dir()
    src_file = tmp_path / "persist.cpp"
    src_file.write_text(PERSIST_PROGRAM)
    exe = tmp_path / "persist"
    r = subprocess.run(["g++", "-std=c++14", f"-I{INCLUDE}", str(src_file), "-o", str(exe), f"-L{lib}",
                        "-lendgraph_gb300", f"-Wl,-rpath,{lib}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    V, E = 30_000, 300_000
    s, d, _ = oracle.rmat(V, E, 71)
    gfile = tmp_path / "g.bin"
    _write_edges(str(gfile), s, d)
    out = tmp_path / "pr.bin"
    r = subprocess.run([str(exe), str(gfile), str(V), str(out)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"size={4 * V} same=1 same_d=1 size_d={8 * V} refused=1" in r.stdout, r.stdout
    outd, _ = oracle.degrees(s, d, V)
    csc = oracle.build_csc(s, d, None, V, np.array([0, V], np.uint32))
    pr = np.fromfile(out, np.float32)
    assert pr.size == V
    assert rel_l1(pr, oracle.pagerank(csc["off"][0], csc["adj"], outd, V, 20, 0.85)) <= 1e-6
