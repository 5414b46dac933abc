"""endgraph_gb300 -- EndGraph preprocessing and the Gemini process_edges toolkits on one GB300.

Python binding of ``libendgraph_gb300.so`` (C ABI: ``include/endgraph_gb300.h``) via ctypes.
``Graph`` mirrors the reference's ``Graph<EdgeData>`` (core/graph.hpp:100): construct with eta,
``load_directed`` / ``load_undirected_from_directed``, then the toolkits.  Buffers may be numpy
arrays (host memory, copied inside the call) or CUDA torch tensors (device memory).

There is no CPU path: every call runs the CUDA kernels of the shared library, and importing
functionality fails loudly when the library is missing or no GPU is present.
"""
from __future__ import annotations

import ctypes
import functools
import os
import sys

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = _build.LIB

EG_HOST, EG_DEVICE = 0, 1
EG_OPT_BFS_DIRECTION, EG_OPT_DENSE_DIVISOR, EG_OPT_CUDA_GRAPH = 1, 2, 3
EG_OPT_PULL_BLOCKS_PER_SM, EG_OPT_BATCH_WIDTH, EG_OPT_SSSP_DELTA, EG_OPT_PR_RELABEL = 4, 5, 6, 7
EG_OPT_MAX_ITERATIONS, EG_OPT_BATCH_LAUNCH, EG_OPT_BATCH_DIVISOR, EG_OPT_BUILD_LAUNCH = 8, 9, 10, 11
STATUS = {0: "EG_OK", 1: "EG_ERR_INVALID", 2: "EG_ERR_CUDA", 3: "EG_ERR_NOMEM", 4: "EG_ERR_STATE",
          5: "EG_ERR_TIMEOUT", 6: "EG_ERR_HOST_CALLBACK", 7: "EG_ERR_UNSUPPORTED"}


class EndGraphError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("eta", ctypes.c_uint64), ("partitions", ctypes.c_int32), ("sub_partitions", ctypes.c_int32),
                ("max_iterations", ctypes.c_int32), ("device", ctypes.c_int32), ("stream", ctypes.c_void_p)]


class Info(ctypes.Structure):
    _fields_ = [("V", ctypes.c_uint32), ("partitions", ctypes.c_uint32), ("E", ctypes.c_uint64),
                ("ncompressed", ctypes.c_uint64), ("weighted", ctypes.c_int32), ("built_csr", ctypes.c_int32),
                ("built_csc", ctypes.c_int32), ("symmetric", ctypes.c_int32)]


class Tuning(ctypes.Structure):
    _fields_ = [("bfs_direction", ctypes.c_int32), ("dense_divisor", ctypes.c_int32),
                ("pull_blocks_per_sm", ctypes.c_int32), ("cuda_graph", ctypes.c_int32), ("batch_width", ctypes.c_int32),
                ("batch_divisor", ctypes.c_int32), ("bfs_ms", ctypes.c_double), ("pull_sweep_ms", ctypes.c_double),
                ("msbfs_ms_per_root", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("launches", ctypes.c_uint64), ("ms", ctypes.c_double)]


# every exported symbol of include/endgraph_gb300.h with its ctypes signature
_vp, _u32, _u64, _i32, _f32, _f64 = (ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int,
                                      ctypes.c_float, ctypes.c_double)
SIGNATURES = {
    "eg_create": ([_vp, _vp], _i32),
    "eg_destroy": ([_vp], _i32),
    "eg_last_error": ([], ctypes.c_char_p),
    "eg_version": ([], _i32),
    "eg_launch_count": ([], ctypes.c_ulonglong),
    "eg_stream": ([_vp], _vp),
    "eg_sync": ([_vp], _i32),
    "eg_load_edges": ([_vp, _vp, _u64, _u32, _i32, _i32, _i32], _i32),
    "eg_build": ([_vp, _i32, _i32], _i32),
    "eg_load_directed": ([_vp, _vp, _u64, _u32, _i32, _i32], _i32),
    "eg_load_undirected_from_directed": ([_vp, _vp, _u64, _u32, _i32, _i32], _i32),
    "eg_get_info": ([_vp, _vp], _i32),
    "eg_get_partition": ([_vp, _vp, _vp], _i32),
    "eg_get_degrees": ([_vp, _vp, _vp, _i32], _i32),
    "eg_get_csr": ([_vp, _vp], _i32),
    "eg_get_csc": ([_vp, _vp], _i32),
    "eg_copy_csr": ([_vp, _vp, _vp, _vp, _vp, _i32], _i32),
    "eg_copy_csc": ([_vp, _vp, _vp, _vp, _vp, _vp, _i32], _i32),
    "eg_cpbt_partition": ([_vp, _u32, _i32, _i32, _u64, _i32, _i32, _i32, _vp, _vp], _i32),
    "eg_optimal_offset": ([_vp, _u32, _u32, _vp], _i32),
    "eg_cpbt_partition_noalloc": ([_vp, _u32, _i32, _i32, _u64, _i32, _i32, _vp, _vp, _vp], _i32),
    "eg_pagerank": ([_vp, _i32, _f32, _vp, _i32], _i32),
    "eg_bfs": ([_vp, _u32, _vp, _vp, _i32, _vp], _i32),
    "eg_cc": ([_vp, _vp, _i32], _i32),
    "eg_sssp": ([_vp, _u32, _vp, _i32], _i32),
    "eg_last_run": ([_vp, _vp, _vp, _vp, _vp], _i32),
    "eg_set_option": ([_vp, _i32, ctypes.c_int64], _i32),
    "eg_msbfs": ([_vp, _vp, _i32, _vp, _i32, _vp], _i32),
    "eg_sssp_batch": ([_vp, _vp, _i32, _vp, _i32], _i32),
    "eg_load_directed_with_ids": ([_vp, _vp, _u64, _u32, _i32], _i32),
    "eg_ppr": ([_vp, _vp, _vp, _i32, _f32, _i32, _vp, _i32], _i32),
    "eg_ppr_backward": ([_vp, _vp, _vp, _i32, _f32, _i32, _vp, _vp, _i32], _i32),
    "eg_bfs_many": ([_vp, _vp, _i32, _vp, _i32, _vp], _i32),
    "eg_autotune": ([_vp, _vp, _i32, _vp], _i32),
    "eg_load_graph_batch": ([_vp, _vp, _i32, _vp, _vp, _i32, _i32], _i32),
    "eg_get_graph_batch": ([_vp, _vp, _vp], _i32),
    "eg_msbfs_graphs": ([_vp, _vp, _i32, _vp, _i32, _vp], _i32),
    "eg_sssp_graphs": ([_vp, _vp, _i32, _vp, _i32], _i32),
    "eg_generate_rmat": ([_vp, _i32, _u64, _u32, _f64, _f64, _f64, _u64, _i32, _f32, _f32, _vp], _i32),
    "eg_profile_enable": ([_vp, _i32], _i32),
    "eg_profile_reset": ([_vp], _i32),
    "eg_profile_read": ([_vp, _vp, _i32, _vp], _i32),
    "eg_selftest_bounded_wait": ([_vp, _u32], _i32),
    "eg_selftest_grid_barrier": ([_vp, _u32], _i32),
    "eg_load_file": ([_vp, ctypes.c_char_p, _u32, _i32, _i32], _i32),
    "eg_load_directed_file": ([_vp, ctypes.c_char_p, _u32, _i32], _i32),
}

_lib = None


def load_library(path: str | None = None, build_if_missing: bool = False):
    """Load libendgraph_gb300.so (raises if it is absent and not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise EndGraphError(1, f"{path} is missing: run `python -m endgraph_gb300.build`")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(status):
    if status != 0:
        msg = load_library().eg_last_error()
        raise EndGraphError(status, msg.decode() if msg else "")


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _buf(x):
    """(pointer, where) of a numpy array or CUDA torch tensor; (None, host) for None."""
    if x is None:
        return None, EG_HOST
    if _is_torch(x):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return ctypes.c_void_p(x.data_ptr()), (EG_DEVICE if x.is_cuda else EG_HOST)
    if not x.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return ctypes.c_void_p(x.ctypes.data), EG_HOST


def _to_device_u32(a, like):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).to(like.device)


def pack_edges(src, dst, w=None):
    """Reference binary records (core/type.hpp:29-43): u32 src, u32 dst [, f32 w], packed."""
    E = len(src)
    if w is None:
        rec = np.empty((E, 2), np.uint32)
        rec[:, 0] = src
        rec[:, 1] = dst
    else:
        rec = np.empty((E, 3), np.uint32)
        rec[:, 0] = src
        rec[:, 1] = dst
        rec[:, 2] = np.asarray(w, np.float32).view(np.uint32)
    return rec


def _torch_ordered(fn):
    """Order the handle's stream after torch's current stream when a CUDA tensor is passed: the
    library runs on its own stream, and a tensor just written by torch (or still read by it) must be
    complete before the library touches it."""
    @functools.wraps(fn)
    def wrapped(self, *args, **kw):
        self._order_after_torch(list(args) + list(kw.values()))
        return fn(self, *args, **kw)
    return wrapped


class Graph:
    """Graph<EdgeData> on one GPU (core/graph.hpp:100-1819)."""

    def _order_after_torch(self, values):
        torch = sys.modules.get("torch")
        if torch is None:
            return
        for x in values:
            if isinstance(x, torch.Tensor) and x.is_cuda:
                ev = torch.cuda.Event()
                ev.record(torch.cuda.current_stream(x.device))
                torch.cuda.ExternalStream(self.stream, device=x.device).wait_event(ev)
                return

    def __init__(self, eta=1, partitions=1, sub_partitions=1, max_iterations=20, device=0, stream=None):
        L = load_library()
        self._L = L
        cfg = Config(eta, partitions, sub_partitions, max_iterations, device, stream)
        h = ctypes.c_void_p()
        _check(L.eg_create(ctypes.byref(h), ctypes.byref(cfg)))
        self.h = h
        self.partitions = partitions
        self.sub_partitions = sub_partitions

    def close(self):
        if getattr(self, "h", None):
            self._L.eg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- loading / preprocessing ----------------------------------------------------------------
    @staticmethod
    def _records(edges):
        if _is_torch(edges):
            rec = edges.shape[-1] * 4 if edges.dim() == 2 else None
            n = edges.shape[0]
            return edges, n, rec
        edges = np.ascontiguousarray(edges)
        return edges, edges.shape[0], edges.shape[1] * 4

    @_torch_ordered
    def load_edges(self, edges, V, symmetric=False):
        edges, E, rec = self._records(edges)
        p, where = _buf(edges)
        _check(self._L.eg_load_edges(self.h, p, E, V, rec, int(symmetric), where))

    def load_file(self, path, V, edge_bytes=8, symmetric=False):
        """Binary records {u32 src, u32 dst[, f32 w]} from a file (preload_graph_file)."""
        _check(self._L.eg_load_file(self.h, os.fsencode(path), V, edge_bytes, int(symmetric)))

    def load_directed_file(self, path, V, edge_bytes=8):
        """load_directed(path, V) in one call: the file is read and uploaded in parts while the
        first build passes consume them."""
        _check(self._L.eg_load_directed_file(self.h, os.fsencode(path), V, edge_bytes))

    def build(self, csr=True, csc=True):
        _check(self._L.eg_build(self.h, int(csr), int(csc)))

    @_torch_ordered
    def load_directed(self, edges, V):
        edges, E, rec = self._records(edges)
        p, where = _buf(edges)
        _check(self._L.eg_load_directed(self.h, p, E, V, rec, where))

    @_torch_ordered
    def load_undirected_from_directed(self, edges, V):
        edges, E, rec = self._records(edges)
        p, where = _buf(edges)
        _check(self._L.eg_load_undirected_from_directed(self.h, p, E, V, rec, where))

    def info(self):
        i = Info()
        _check(self._L.eg_get_info(self.h, ctypes.byref(i)))
        return i

    @property
    def stream(self):
        return self._L.eg_stream(self.h)

    def sync(self):
        _check(self._L.eg_sync(self.h))

    def partition(self):
        i = self.info()
        po = np.empty(i.partitions + 1, np.uint32)
        lo = np.empty(i.partitions * (self.sub_partitions + 1), np.uint32)
        _check(self._L.eg_get_partition(self.h, _buf(po)[0], _buf(lo)[0]))
        return po, lo.reshape(i.partitions, self.sub_partitions + 1)

    def degrees(self):
        V = self.info().V
        out = np.empty(V, np.uint32)
        inn = np.empty(V, np.uint32)
        _check(self._L.eg_get_degrees(self.h, _buf(out)[0], _buf(inn)[0], EG_HOST))
        return out, inn

    def csr(self):
        i = self.info()
        P, V, E = i.partitions, i.V, i.E
        off = np.empty(P * (V + 1), np.uint64)
        adj = np.empty(max(E, 1), np.uint32)
        w = np.empty(max(E, 1), np.float32) if i.weighted else None
        bm = np.empty(P * (V // 64 + 1), np.uint64)
        _check(self._L.eg_copy_csr(self.h, _buf(off)[0], _buf(adj)[0], _buf(w)[0], _buf(bm)[0], EG_HOST))
        return dict(off=off.reshape(P, V + 1), adj=adj[:E], w=None if w is None else w[:E],
                    bitmap=bm.reshape(P, V // 64 + 1))

    def csc(self):
        i = self.info()
        P, V, E, n = i.partitions, i.V, i.E, i.ncompressed
        off = np.empty(P * (V + 1), np.uint64)
        adj = np.empty(max(E, 1), np.uint32)
        w = np.empty(max(E, 1), np.float32) if i.weighted else None
        cv = np.empty(max(n, 1), np.uint32)
        ci = np.empty(max(n, 1), np.uint64)
        _check(self._L.eg_copy_csc(self.h, _buf(off)[0], _buf(adj)[0], _buf(w)[0], _buf(cv)[0], _buf(ci)[0],
                                   EG_HOST))
        return dict(off=off.reshape(P, V + 1), adj=adj[:E], w=None if w is None else w[:E], cvert=cv[:n],
                    cidx=ci[:n])

    # ---- toolkits ------------------------------------------------------------------------------
    @_torch_ordered
    def pagerank(self, iterations=20, damping=0.85, out=None):
        if out is None:
            out = np.empty(self.info().V, np.float32)
        p, where = _buf(out)
        _check(self._L.eg_pagerank(self.h, iterations, damping, p, where))
        return out

    @_torch_ordered
    def bfs(self, root, level=None, parent=None, want_parent=True):
        V = self.info().V
        if level is None:
            level = np.empty(V, np.uint32)
        if parent is None and want_parent:
            parent = np.empty(V, np.uint32)
        pl, where = _buf(level)
        pp, _ = _buf(parent)
        reached = ctypes.c_uint64()
        _check(self._L.eg_bfs(self.h, root, pl, pp, where, ctypes.byref(reached)))
        return level, parent

    @_torch_ordered
    def cc(self, label=None):
        if label is None:
            label = np.empty(self.info().V, np.uint32)
        p, where = _buf(label)
        _check(self._L.eg_cc(self.h, p, where))
        return label

    @_torch_ordered
    def sssp(self, root, dist=None):
        if dist is None:
            dist = np.empty(self.info().V, np.float32)
        p, where = _buf(dist)
        _check(self._L.eg_sssp(self.h, root, p, where))
        return dist

    @_torch_ordered
    def load_directed_with_ids(self, edges, V):
        edges, E, rec = self._records(edges)
        if rec != 8:
            raise ValueError("eg_load_directed_with_ids takes {src, dst} records")
        p, where = _buf(edges)
        _check(self._L.eg_load_directed_with_ids(self.h, p, E, V, where))

    @_torch_ordered
    def msbfs(self, roots, levels=None):
        roots = np.ascontiguousarray(roots, np.uint32)
        V = self.info().V
        if levels is None:
            levels = np.empty((len(roots), V), np.uint8)
        p, where = _buf(levels)
        if where == EG_DEVICE:
            import torch
            roots_t = torch.from_numpy(roots.view(np.int32)).to(levels.device)
            rp = _buf(roots_t)[0]
        else:
            rp = _buf(roots)[0]
        e = ctypes.c_uint64()
        _check(self._L.eg_msbfs(self.h, rp, len(roots), p, where, ctypes.byref(e)))
        return levels, e.value

    @_torch_ordered
    def sssp_batch(self, sources, dist=None):
        sources = np.ascontiguousarray(sources, np.uint32)
        V = self.info().V
        if dist is None:
            dist = np.empty((len(sources), V), np.float32)
        p, where = _buf(dist)
        if where == EG_DEVICE:
            import torch
            sp = _buf(torch.from_numpy(sources.view(np.int32)).to(dist.device))[0]
        else:
            sp = _buf(sources)[0]
        _check(self._L.eg_sssp_batch(self.h, sp, len(sources), p, where))
        return dist

    @_torch_ordered
    def ppr(self, weights, seeds, alpha=0.15, iterations=50, out=None):
        """weights and out on the host (numpy) or all on the device (torch)."""
        seeds = np.ascontiguousarray(seeds, np.uint32)
        V = self.info().V
        if out is None:
            out = np.empty((len(seeds), V), np.float32)
        wp, where = _buf(weights)
        op, _ = _buf(out)
        sp = _buf(seeds)[0] if where == EG_HOST else _buf(_to_device_u32(seeds, weights))[0]
        _check(self._L.eg_ppr(self.h, wp, sp, len(seeds), alpha, iterations, op, where))
        return out

    @_torch_ordered
    def ppr_backward(self, weights, seeds, dl_dx, alpha=0.15, iterations=50, dl_dw=None):
        seeds = np.ascontiguousarray(seeds, np.uint32)
        if dl_dw is None:
            dl_dw = np.empty(len(weights), np.float32)
        wp, where = _buf(weights)
        sp = _buf(seeds)[0] if where == EG_HOST else _buf(_to_device_u32(seeds, weights))[0]
        _check(self._L.eg_ppr_backward(self.h, wp, sp, len(seeds), alpha, iterations, _buf(dl_dx)[0], _buf(dl_dw)[0],
                                       where))
        return dl_dw

    @_torch_ordered
    def bfs_many(self, roots, levels=None):
        roots = np.ascontiguousarray(roots, np.uint32)
        p, where = _buf(levels)
        rp = _buf(roots)[0] if where == EG_HOST else _buf(_to_device_u32(roots, levels))[0]
        e = ctypes.c_uint64()
        _check(self._L.eg_bfs_many(self.h, rp, len(roots), p, where, ctypes.byref(e)))
        return levels, e.value

    def autotune(self, sample_roots):
        r = np.ascontiguousarray(sample_roots, np.uint32)
        t = Tuning()
        _check(self._L.eg_autotune(self.h, _buf(r)[0], len(r), ctypes.byref(t)))
        return t.as_dict()

    @_torch_ordered
    def load_graph_batch(self, edges, graph_edges, graph_vertices):
        """edges: all graphs' records back to back; graph_edges[G+1]; graph_vertices[G]."""
        edges, E, rec = self._records(edges)
        p, where = _buf(edges)
        ge = np.ascontiguousarray(graph_edges, np.uint64)
        gv = np.ascontiguousarray(graph_vertices, np.uint32)
        _check(self._L.eg_load_graph_batch(self.h, p, rec, _buf(ge)[0], _buf(gv)[0], len(gv), where))
        self._batch_G = len(gv)

    def graph_batch(self):
        G = self._batch_G
        vo = np.empty(G + 1, np.uint64)
        eo = np.empty(G + 1, np.uint64)
        _check(self._L.eg_get_graph_batch(self.h, _buf(vo)[0], _buf(eo)[0]))
        return vo, eo

    @_torch_ordered
    def msbfs_graphs(self, roots, per_graph, levels=None):
        roots = np.ascontiguousarray(roots, np.uint32)
        if levels is None:
            levels = np.empty((self.info().V, 64), np.uint8)
        p, where = _buf(levels)
        rp = _buf(roots)[0] if where == EG_HOST else _buf(_to_device_u32(roots, levels))[0]
        e = ctypes.c_uint64()
        _check(self._L.eg_msbfs_graphs(self.h, rp, per_graph, p, where, ctypes.byref(e)))
        return levels, e.value

    @_torch_ordered
    def sssp_graphs(self, sources, per_graph, dist=None):
        sources = np.ascontiguousarray(sources, np.uint32)
        if dist is None:
            dist = np.empty((self.info().V, 64), np.float32)
        p, where = _buf(dist)
        sp = _buf(sources)[0] if where == EG_HOST else _buf(_to_device_u32(sources, dist))[0]
        _check(self._L.eg_sssp_graphs(self.h, sp, per_graph, p, where))
        return dist

    def set_option(self, option, value):
        _check(self._L.eg_set_option(self.h, option, value))

    def last_run(self):
        e = ctypes.c_uint64()
        it, pu, pl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(self._L.eg_last_run(self.h, ctypes.byref(e), ctypes.byref(it), ctypes.byref(pu), ctypes.byref(pl)))
        return dict(edges=e.value, iterations=it.value, push=pu.value, pull=pl.value)

    # ---- profiling ------------------------------------------------------------------------------
    def profile(self, enable=True):
        _check(self._L.eg_profile_enable(self.h, int(enable)))

    def profile_reset(self):
        _check(self._L.eg_profile_reset(self.h))

    def selftest_bounded_wait(self, spin_cap=1000):
        """Status of a look-back scan whose wait is made to run out (EG_ERR_TIMEOUT expected)."""
        return self._L.eg_selftest_bounded_wait(self.h, spin_cap)

    def selftest_grid_barrier(self, spin_cap=1000):
        """Status of a cooperative launch whose grid barrier is made to run out (EG_ERR_TIMEOUT
        expected)."""
        return self._L.eg_selftest_grid_barrier(self.h, spin_cap)

    def profile_read(self):
        n = ctypes.c_int()
        _check(self._L.eg_profile_read(self.h, None, 0, ctypes.byref(n)))
        arr = (KernelStat * max(n.value, 1))()
        _check(self._L.eg_profile_read(self.h, arr, n.value, ctypes.byref(n)))
        return {arr[i].name.decode(): (arr[i].launches, arr[i].ms) for i in range(n.value)}


def cpbt_partition(deg, V, P, S=1, eta=1, max_iterations=20, dense=True):
    """assign_vertices boundaries (core/graph.hpp:662-792) computed on the GPU."""
    L = load_library()
    po = np.empty(P + 1, np.uint32)
    lo = np.empty(P * (S + 1), np.uint32)
    p, where = _buf(deg)
    _check(L.eg_cpbt_partition(p, V, P, S, eta, max_iterations, int(dense), where, _buf(po)[0], _buf(lo)[0]))
    return po, lo.reshape(P, S + 1)


def optimal_offset(a, k):
    """optimal_offset(a, n, k) (core/graph.hpp:597-626) on the GPU."""
    L = load_library()
    a = np.ascontiguousarray(a, np.uint64)
    out = np.empty(k + 1, np.uint32)
    _check(L.eg_optimal_offset(_buf(a)[0] if len(a) else None, len(a), k, _buf(out)[0]))
    return out


def generate_rmat(out, V, E, seed, a=0.57, b=0.19, c=0.19, permute=True, weights=None, stream=None):
    """Fill a CUDA tensor of shape (E, 2) or (E, 3) (uint32/int32 storage) with R-MAT records."""
    L = load_library()
    rec = out.shape[1] * 4
    lo, hi = weights or (0.0, 1.0)
    if stream is None:  # torch's stream, so that torch and the library see the records in order
        import torch
        stream = ctypes.c_void_p(torch.cuda.current_stream(out.device).cuda_stream)
    _check(L.eg_generate_rmat(ctypes.c_void_p(out.data_ptr()), rec, E, V, a, b, c, seed, int(permute), lo, hi,
                              stream))
    return out
