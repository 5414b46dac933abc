"""CPU oracle for EndGraph's preprocessing and the Gemini toolkits -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg (and its
``--impl reference`` arm) may import this package; the product (``endgraph_gb300``) never does.

Two checkers live here:

* ``libeg_oracle.so`` -- ``eg_oracle.c``, a plain-C restatement of the reference algorithm, each
  function citing the ``core/graph.hpp`` / ``toolkits/*.cpp`` lines it follows;
* ``_ref/libeg_ref.so`` -- the reference's own engine compiled at one rank by ``build_ref.sh``
  (present where the reference sources were available at build time).

The restatement is pinned against the reference build and against ``tests/golden/`` vectors.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libeg_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libeg_ref.so")
UNREACHED = 0xFFFFFFFF

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class RmatParams(ctypes.Structure):
    """Mirror of ``eg_rmat_params`` (include/endgraph_rmat.h)."""

    _fields_ = [
        ("seed", ctypes.c_uint64), ("E", ctypes.c_uint64), ("V", ctypes.c_uint32),
        ("scale", ctypes.c_uint32), ("ta", ctypes.c_uint32), ("tab", ctypes.c_uint32),
        ("tabc", ctypes.c_uint32), ("permute", ctypes.c_uint32), ("w_lo", ctypes.c_float),
        ("w_hi", ctypes.c_float),
    ]


def rmat_params(V, E, seed, a=0.57, b=0.19, c=0.19, permute=True, w_lo=0.0, w_hi=1.0):
    scale = 0
    while scale < 32 and (1 << scale) < V:
        scale += 1
    return RmatParams(seed, E, V, scale, int(a * 4294967296.0), int((a + b) * 4294967296.0),
                      int((a + b + c) * 4294967296.0), 1 if permute else 0, w_lo, w_hi)


def reference_dir() -> str | None:
    """Directory of the reference checkout: $EG_REFERENCE_DIR, else the one build_ref.sh compiled
    from (recorded in _ref/REFERENCE_DIR); None when neither exists on this machine."""
    cand = [os.environ.get("EG_REFERENCE_DIR")]
    rec = os.path.join(HERE, "_ref", "REFERENCE_DIR")
    if os.path.exists(rec):
        with open(rec) as f:
            cand.append(f.read().strip())
    for d in cand:
        if d and os.path.isfile(os.path.join(d, "core", "graph.hpp")):
            return d
    return None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "eg_oracle.c")
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "eg_oracle.h"))):
        tmp = ORACLE_SO + ".tmp"
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC",
                               "-shared", src, "-o", tmp, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref() -> str | None:
    """Build oracle/_ref/libeg_ref.so from the reference sources; None when they are absent."""
    r = subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], capture_output=True, text=True)
    return REF_SO if r.returncode == 0 and os.path.exists(REF_SO) else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(ORACLE_SO)
        L.ora_rmat.argtypes = [ctypes.POINTER(RmatParams), ctypes.c_uint64, ctypes.c_uint64, _u32p, _u32p,
                               ctypes.c_void_p]
        L.ora_degrees.argtypes = [_u32p, _u32p, ctypes.c_uint64, ctypes.c_uint32, _u32p, _u32p]
        L.ora_page_weights.argtypes = [_u32p, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                       ctypes.c_int, _u64p]
        L.ora_optimal_offset.argtypes = [_u64p, ctypes.c_uint32, ctypes.c_uint32, _u32p]
        L.ora_cpbt.argtypes = [_u32p, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                               ctypes.c_int, _u32p, _u32p]
        L.ora_build_csr.argtypes = [_u32p, _u32p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int,
                                    _u32p, _u64p, _u64p, _u32p, ctypes.c_void_p, _u64p]
        L.ora_build_csc.argtypes = [_u32p, _u32p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int,
                                    _u32p, _u64p, _u64p, _u32p, ctypes.c_void_p, _u64p, _u32p, _u64p,
                                    ctypes.c_uint64]
        L.ora_build_csc.restype = ctypes.c_uint64
        L.ora_pagerank.argtypes = [_u64p, _u32p, _u32p, ctypes.c_uint32, ctypes.c_int, ctypes.c_double, _f64p]
        L.ora_bfs_levels.argtypes = [_u64p, _u32p, ctypes.c_uint32, ctypes.c_uint32, _u32p]
        L.ora_bfs_check_parents.argtypes = [_u64p, _u32p, ctypes.c_uint32, ctypes.c_uint32, _u32p, _u32p]
        L.ora_bfs_check_parents.restype = ctypes.c_uint64
        L.ora_cc_labels.argtypes = [_u32p, _u32p, ctypes.c_uint64, ctypes.c_uint32, _u32p]
        L.ora_sssp.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32, _f32p]
        L.ora_bc.argtypes = [_u64p, _u32p, ctypes.c_uint32, ctypes.c_uint32, _f64p, _f64p, _u32p]
        L.ora_adjacency_hash.argtypes = [_u32p, _u32p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                         _u64p, _u64p]
        L.ora_list_hash.argtypes = [_u64p, _u32p, ctypes.c_void_p, ctypes.c_uint64, _u64p]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def rmat(V, E, seed, a=0.57, b=0.19, c=0.19, permute=True, weights=None, e0=0):
    """Edges [e0, e0+E) of the seeded R-MAT stream; weights=(lo, hi) adds float32 weights."""
    p = rmat_params(V, E, seed, a, b, c, permute, *(weights or (0.0, 1.0)))
    src = np.empty(E, np.uint32)
    dst = np.empty(E, np.uint32)
    w = np.empty(E, np.float32) if weights else None
    lib().ora_rmat(ctypes.byref(p), e0, E, src, dst, _ptr(w))
    return src, dst, w


def degrees(src, dst, V):
    out = np.empty(V, np.uint32)
    inn = np.empty(V, np.uint32)
    lib().ora_degrees(src, dst, len(src), V, out, inn)
    return out, inn


def page_weights(deg, V, P, eta, max_iterations, dense):
    pages = (V + 4095) // 4096
    out = np.empty(max(pages, 1), np.uint64)
    lib().ora_page_weights(deg, V, P, eta, max_iterations, 1 if dense else 0, out)
    return out[:pages]


def optimal_offset(a, k):
    a = np.ascontiguousarray(a, np.uint64)
    out = np.empty(k + 1, np.uint32)
    lib().ora_optimal_offset(a if len(a) else np.zeros(1, np.uint64), len(a), k, out)
    return out


def cpbt(deg, V, P, S=1, eta=1, max_iterations=20, dense=True):
    poff = np.empty(P + 1, np.uint32)
    loff = np.empty(P * (S + 1), np.uint32)
    lib().ora_cpbt(np.ascontiguousarray(deg, np.uint32), V, P, S, eta, max_iterations, 1 if dense else 0, poff,
                   loff)
    return poff, loff.reshape(P, S + 1)


def build_csr(src, dst, w, V, poff):
    P = len(poff) - 1
    E = len(src)
    part_start = np.empty(P + 1, np.uint64)
    off = np.empty(P * (V + 1), np.uint64)
    col = np.empty(max(E, 1), np.uint32)
    cw = np.empty(max(E, 1), np.float32) if w is not None else None
    bitmap = np.empty(P * (V // 64 + 1), np.uint64)
    lib().ora_build_csr(src, dst, _ptr(w), E, V, P, np.ascontiguousarray(poff, np.uint32), part_start, off, col,
                        _ptr(cw), bitmap)
    return dict(part_start=part_start, off=off.reshape(P, V + 1), adj=col[:E], w=None if cw is None else cw[:E],
                bitmap=bitmap.reshape(P, V // 64 + 1))


def build_csc(src, dst, w, V, poff):
    P = len(poff) - 1
    E = len(src)
    part_start = np.empty(P + 1, np.uint64)
    off = np.empty(P * (V + 1), np.uint64)
    col = np.empty(max(E, 1), np.uint32)
    cw = np.empty(max(E, 1), np.float32) if w is not None else None
    cstart = np.empty(P + 1, np.uint64)
    cap = min(E + P, P * (V + 1)) + 1
    cvert = np.empty(cap, np.uint32)
    cidx = np.empty(cap, np.uint64)
    n = lib().ora_build_csc(src, dst, _ptr(w), E, V, P, np.ascontiguousarray(poff, np.uint32), part_start, off,
                            col, _ptr(cw), cstart, cvert, cidx, cap)
    assert n <= cap
    return dict(part_start=part_start, off=off.reshape(P, V + 1), adj=col[:E], w=None if cw is None else cw[:E],
                cstart=cstart, cvert=cvert[:n], cidx=cidx[:n])


def pagerank(csc_off, csc_src, outdeg, V, iterations=20, damping=0.85):
    out = np.empty(max(V, 1), np.float64)
    lib().ora_pagerank(np.ascontiguousarray(csc_off, np.uint64), csc_src, outdeg, V, iterations, damping, out)
    return out[:V]


def bc(csr_off, csr_dst, V, root):
    """(sigma, delta, level) of single-source betweenness from root (Brandes)."""
    sigma = np.empty(V, np.float64)
    delta = np.empty(V, np.float64)
    level = np.empty(V, np.uint32)
    lib().ora_bc(np.ascontiguousarray(csr_off, np.uint64), csr_dst, V, root, sigma, delta, level)
    return sigma, delta, level


def bfs_levels(csr_off, csr_dst, V, root):
    out = np.empty(V, np.uint32)
    lib().ora_bfs_levels(np.ascontiguousarray(csr_off, np.uint64), csr_dst, V, root, out)
    return out


def bfs_check_parents(csr_off, csr_dst, V, root, level, parent):
    return int(lib().ora_bfs_check_parents(np.ascontiguousarray(csr_off, np.uint64), csr_dst, V, root,
                                           np.ascontiguousarray(level, np.uint32),
                                           np.ascontiguousarray(parent, np.uint32)))


def cc_labels(src, dst, V):
    out = np.empty(V, np.uint32)
    lib().ora_cc_labels(src, dst, len(src), V, out)
    return out


def sssp(csr_off, csr_dst, csr_w, V, root):
    out = np.empty(V, np.float32)
    lib().ora_sssp(np.ascontiguousarray(csr_off, np.uint64), csr_dst, csr_w, V, root, out)
    return out


def adjacency_hash(src, dst, w, V):
    hout = np.empty(V, np.uint64)
    hin = np.empty(V, np.uint64)
    lib().ora_adjacency_hash(src, dst, _ptr(w), len(src), V, hout, hin)
    return hout, hin


def list_hash(off, adj, w=None):
    """Per-list signature of a CSR/CSC (off[n+1], adj): equal to adjacency_hash's hout (CSR) or
    hin (CSC) for the edge list it was built from, whatever the order inside each list."""
    off = np.ascontiguousarray(off, np.uint64)
    n = len(off) - 1
    out = np.empty(max(n, 1), np.uint64)
    lib().ora_list_hash(off, np.ascontiguousarray(adj, np.uint32), _ptr(w), n, out)
    return out[:n]


def sorted_lists(off, adj, w=None):
    """Per-list sort (by neighbour, then weight bits) for order-independent comparison."""
    off = np.asarray(off, np.int64)
    n = len(off) - 1
    seg = np.repeat(np.arange(n, dtype=np.int64), np.diff(off))
    keys = [adj[off[0]:off[-1]].astype(np.int64)]
    if w is not None:
        keys.insert(0, w[off[0]:off[-1]].view(np.uint32).astype(np.int64))
    order = np.lexsort(tuple(keys) + (seg,))
    a = adj[off[0]:off[-1]][order]
    return a, (None if w is None else w[off[0]:off[-1]][order])


class Reference:
    """The reference's own engine at one rank (oracle/_ref/libeg_ref.so)."""

    _L = None

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(REF_SO)

    @classmethod
    def lib(cls):
        if cls._L is None:
            L = ctypes.CDLL(REF_SO)
            vp = ctypes.c_void_p
            L.ref_threads.restype = ctypes.c_int
            L.ref_optimal_offset.argtypes = [_u64p, ctypes.c_uint32, ctypes.c_uint32, _u32p]
            L.ref_cpbt.argtypes = [_u32p, _u32p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_int, _u32p, _u32p, vp]
            L.ref_create.argtypes = [vp, vp, vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int]
            L.ref_create.restype = vp
            L.ref_build.argtypes = [vp]
            L.ref_build.restype = ctypes.c_double
            L.ref_destroy.argtypes = [vp]
            L.ref_num_edges.argtypes = [vp]
            L.ref_num_edges.restype = ctypes.c_uint64
            L.ref_num_compressed.argtypes = [vp]
            L.ref_num_compressed.restype = ctypes.c_uint64
            L.ref_get_structure.argtypes = [vp] * 13
            L.ref_list_hashes.argtypes = [vp, vp, vp]
            L.ref_pagerank.argtypes = [vp, ctypes.c_int, vp]
            L.ref_pagerank.restype = ctypes.c_double
            L.ref_bfs.argtypes = [vp, ctypes.c_uint32, vp, vp]
            L.ref_bfs.restype = ctypes.c_double
            L.ref_cc.argtypes = [vp, vp, vp]
            L.ref_cc.restype = ctypes.c_double
            L.ref_sssp.argtypes = [vp, ctypes.c_uint32, vp]
            L.ref_sssp.restype = ctypes.c_double
            cls._L = L
        return cls._L

    def __init__(self, src, dst, w, V, symmetric=False, eta=1, max_iterations=20, quiet=True):
        self.V = V
        self.src, self.dst, self.w = src, dst, w
        self.h = self.lib().ref_create(_ptr(src), _ptr(dst), _ptr(w), len(src), V, int(symmetric), eta,
                                       max_iterations, int(quiet))
        self.prep_time = None

    def build(self):
        self.prep_time = self.lib().ref_build(self.h)
        return self.prep_time

    def close(self):
        if self.h:
            self.lib().ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def structure(self):
        L = self.lib()
        E = int(L.ref_num_edges(self.h))
        V = self.V
        nc = int(L.ref_num_compressed(self.h))
        wt = self.w is not None
        d = dict(degree=np.empty(V, np.uint32), partition_offset=np.empty(2, np.uint32),
                 csr_src=np.empty(E, np.uint32), csr_dst=np.empty(E, np.uint32),
                 csr_w=np.empty(E, np.float32) if wt else None, csr_index=np.empty(V + 1, np.uint64),
                 csr_bitmap=np.empty(V // 64 + 1, np.uint64), csc_src=np.empty(E, np.uint32),
                 csc_dst=np.empty(E, np.uint32), csc_w=np.empty(E, np.float32) if wt else None,
                 cvert=np.empty(nc, np.uint32), cidx=np.empty(nc, np.uint64))
        L.ref_get_structure(self.h, *[_ptr(d[k]) for k in (
            "degree", "partition_offset", "csr_src", "csr_dst", "csr_w", "csr_index", "csr_bitmap", "csc_src",
            "csc_dst", "csc_w", "cvert", "cidx")])
        return d

    def summary(self):
        """The vertex-sized parts of the reference's structures (degrees, partition offsets, CSR
        index and source bitmap, compressed CSC index) and per-vertex list signatures of its CSR
        (hout) and CSC (hin): the whole structure without copying the edge-sized lists."""
        L = self.lib()
        V = self.V
        nc = int(L.ref_num_compressed(self.h))
        d = dict(degree=np.empty(V, np.uint32), partition_offset=np.empty(2, np.uint32),
                 csr_index=np.empty(V + 1, np.uint64), csr_bitmap=np.empty(V // 64 + 1, np.uint64),
                 cvert=np.empty(nc, np.uint32), cidx=np.empty(nc, np.uint64))
        L.ref_get_structure(self.h, _ptr(d["degree"]), _ptr(d["partition_offset"]), None, None, None,
                            _ptr(d["csr_index"]), _ptr(d["csr_bitmap"]), None, None, None, _ptr(d["cvert"]),
                            _ptr(d["cidx"]))
        d["hout"] = np.empty(V, np.uint64)
        d["hin"] = np.empty(V, np.uint64)
        L.ref_list_hashes(self.h, _ptr(d["hout"]), _ptr(d["hin"]))
        return d

    def pagerank(self, iterations=20):
        out = np.empty(self.V, np.float64)
        t = self.lib().ref_pagerank(self.h, iterations, _ptr(out))
        return out, t

    def bfs(self, root, want_levels=True):
        level = np.empty(self.V, np.uint32) if want_levels else None
        parent = np.empty(self.V, np.uint32)
        t = self.lib().ref_bfs(self.h, root, _ptr(level), _ptr(parent))
        return level, parent, t

    def cc(self):
        label = np.empty(self.V, np.uint32)
        it = ctypes.c_int(0)
        t = self.lib().ref_cc(self.h, _ptr(label), ctypes.byref(it))
        return label, it.value, t

    def sssp(self, root):
        dist = np.empty(self.V, np.float32)
        t = self.lib().ref_sssp(self.h, root, _ptr(dist))
        return dist, t

    @classmethod
    def optimal_offset(cls, a, k):
        a = np.ascontiguousarray(a, np.uint64)
        out = np.empty(k + 1, np.uint32)
        cls.lib().ref_optimal_offset(a if len(a) else np.zeros(1, np.uint64), len(a), k, out)
        return out

    @classmethod
    def cpbt(cls, src, dst, V, P, S=1, eta=1, max_iterations=20, dense=True):
        poff = np.empty(P + 1, np.uint32)
        loff = np.empty(P * (S + 1), np.uint32)
        deg = np.empty(V, np.uint32)
        cls.lib().ref_cpbt(src, dst, len(src), V, P, S, eta, max_iterations, 1 if dense else 0, poff, loff,
                           _ptr(deg))
        return poff, loff.reshape(P, S + 1), deg
